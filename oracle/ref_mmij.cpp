// ORACLE -- test infrastructure only.  Reaction field of the MMIJ basis,
// restated from the reference in its expression order:
//   rect_rf1.f90:19-161   ENERGY, RECTBOX: Legendre products P_a(x s_x)
//                          P_b(y s_y) P_c(z s_z) of the mobile ions in the
//                          region (centred at the origin), coef, mq = M coef
//                          rfscal, egsbpb = celec sum coef mq / 2, forces
//   rect_rf0.f90:19-114   INTERACT, RECTBOX: E(coef) - E(coef without j)
//   sphe_rf1.f90, sphe_rf0.f90 with rpowerl2, cosmphi2, sinmphi2, alpol2,
//   dalpol2: the same for the SPHERE multipole basis
//   rect_norm.f90, sphe_norm.f90, sphe_svpol.f90, factori.f90: the basis
// Where the reference's arithmetic is defined it is kept, quirks included:
// the region of RECTBOX is [-1/s, 1/s] whatever the given bounds' centre;
// sphe_rf1 forms cos/sin(phi) with 10/sin(theta) (sphe_rf0 with
// 1/sin(theta)), and its forces use the 10/sin(theta) of the last ion in
// the sphere.  Where it is not -- alpol2/dalpol2 declare the arrays of
// sphe_rf1 with other bounds (the element layouts agree only at nmpol 25),
// P_l^m with m > l is read without being set, and INTERACT of a particle
// outside the region or not a mobile ion reads its basis values unset --
// this restatement uses one (l, m) layout, P_l^m = 0 for m > l, and no
// contribution from a particle outside the region or not mobile.
#include <cmath>

#include "ref_state.h"

namespace bref {

// factori.f90
static double factori(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f = f * i;
  return f;
}

// rect_norm.f90 / sphe_norm.f90 / sphe_svpol.f90 (0-based vectors of ntpol)
void mmij_basis(Mmij &m) {
  m.bnorm.assign(m.ntpol, 0.0);
  if (m.rect) {
    const double ilxyz = m.xscal * m.yscal * m.zscal * 0.125;
    for (int n = 0; n < m.ntpol; ++n)
      m.bnorm[n] = std::sqrt((2.0 * m.lstpx[n] + 1.0) * (2.0 * m.lstpy[n] + 1.0) *
                             (2.0 * m.lstpz[n] + 1.0) * ilxyz);
    return;
  }
  m.lstpl.clear();
  m.lstpm.clear();
  for (int l = 0; l < m.nmpol; ++l) {
    m.lstpl.push_back(l);
    m.lstpm.push_back(0);
    for (int mm = 1; mm <= l; ++mm) {
      m.lstpl.push_back(l);
      m.lstpm.push_back(mm);
      m.lstpl.push_back(l);
      m.lstpm.push_back(-mm);
    }
  }
  int norder = 0;
  const double sr2 = m.srdist * m.srdist;
  double rpart = sr2 * m.srdist;
  const double itwopi = 1.0 / twopi;
  double lpart = 1.5 * itwopi;
  const double ipi = 0.5 * itwopi;
  m.bnorm[norder] = std::sqrt(lpart / rpart);
  for (int l = 1; l <= m.nmpol - 1; ++l) {
    lpart = (2.0 * l + 1.0) * (2.0 * l + 3.0) * ipi;
    rpart = rpart * sr2;
    m.bnorm[++norder] = std::sqrt(lpart / rpart);
    lpart = (2.0 * l + 1.0) * (2.0 * l + 3.0) * itwopi;
    for (int mm = 1; mm <= l; ++mm) {
      const double up = factori(l - mm), dn = factori(l + mm);
      ++norder;
      m.bnorm[norder] = std::sqrt(lpart * up / (rpart * dn));
      ++norder;
      m.bnorm[norder] = m.bnorm[norder - 1];
    }
  }
}

namespace {

struct LegRect {
  std::vector<double> lx, ly, lz;  // P_0..P_{n-1}
};

// rect_rf1.f90:33-55: the Legendre values of one position
LegRect legendre_rect(const Mmij &m, double xg, double yg, double zg) {
  LegRect L;
  const double xs[3] = {m.xscal * xg, m.yscal * yg, m.zscal * zg};
  const int np[3] = {m.xnpol, m.ynpol, m.znpol};
  std::vector<double> *out[3] = {&L.lx, &L.ly, &L.lz};
  for (int a = 0; a < 3; ++a) {
    std::vector<double> &v = *out[a];
    v.assign(std::max(np[a], 3), 0.0);
    v[0] = 1.0;
    v[1] = xs[a];
    v[2] = 0.5 * (3.0 * xs[a] * xs[a] - 1.0);
    // lpol(n+1) = ((2n-1) x lpol(n) - (n-1) lpol(n-1)) / n, 1-based
    for (int n = 3; n <= np[a] - 1; ++n)
      v[n] = ((2.0 * n - 1) * xs[a] * v[n - 1] - (n - 1.0) * v[n - 2]) / n;
  }
  return L;
}

bool in_rect(const Mmij &m, double xg, double yg, double zg) {
  return xg >= m.xmin && xg <= m.xmax && yg >= m.ymin && yg <= m.ymax && zg >= m.zmin &&
         zg <= m.zmax;
}

// The spherical tables of one position (sphe_rf1.f90:37-64): r^l, cos(m
// phi), sin(m phi), P_l^m and dP_l^m/dx in the (l, m) layout.
struct LegSphe {
  double r = 0, ct = 0, st = 0, cp = 0, sp = 0, ist = 0;
  std::vector<double> ar, ac, as, ap, adp;  // ap/adp [(lmax+2) x (mmax+2)]
  int w = 0;
  double P(int l, int mm) const { return ap[(size_t)l * w + mm]; }
  double dP(int l, int mm) const { return adp[(size_t)l * w + mm]; }
};

LegSphe legendre_sphe(const Mmij &m, double xd, double yd, double zd, double istnum) {
  LegSphe S;
  const int lmax = m.nmpol - 1, mmax = lmax;
  const double r2 = xd * xd + yd * yd + zd * zd;
  S.r = std::sqrt(r2);
  const double ir = 1.0 / S.r;
  S.ct = zd * ir;
  S.st = std::sqrt(1.0 - S.ct * S.ct);
  S.ist = istnum / S.st;
  S.cp = xd * ir * S.ist;
  S.sp = yd * ir * S.ist;
  if (r2 < rsmall) {  // at the origin
    S.ct = S.st = S.cp = S.sp = 0.0;
  } else if (xd > -rsmall && xd < rsmall && yd > -rsmall && yd < rsmall) {  // z axis
    S.ct = zd < 0.0 ? -1.0 : 1.0;
    S.cp = S.sp = 0.0;
  } else if (zd > -rsmall && zd < rsmall) {  // xy plane
    S.ct = 0.0;
    S.cp = xd * ir;
    S.sp = yd * ir;
  }
  // rpowerl2
  S.ar.assign(lmax + 1, 0.0);
  S.ar[0] = 1.0;
  for (int i = 1; i <= lmax; ++i) S.ar[i] = S.ar[i - 1] * S.r;
  // cosmphi2 / sinmphi2 (they fill orders 0..3 whatever mmax is)
  const int mc = std::max(mmax, 3);
  S.ac.assign(mc + 1, 0.0);
  S.as.assign(mc + 1, 0.0);
  S.ac[0] = 1.0;
  S.ac[1] = S.cp;
  S.ac[2] = 2.0 * S.cp * S.cp - 1.0;
  S.ac[3] = (2.0 * S.ac[2] - 1.0) * S.cp;
  for (int i = 4; i <= mmax; ++i) S.ac[i] = 2.0 * S.cp * S.ac[i - 1] - S.ac[i - 2];
  S.as[0] = 0.0;
  S.as[1] = S.sp;
  S.as[2] = 2.0 * S.cp * S.sp;
  S.as[3] = 2.0 * S.cp * S.as[2] - S.sp;
  for (int i = 4; i <= mmax; ++i) S.as[i] = 2.0 * S.cp * S.as[i - 1] - S.as[i - 2];
  // alpol2 (P_l^m = 0 for m > l)
  S.w = mmax + 2;
  S.ap.assign((size_t)(lmax + 2) * S.w, 0.0);
  S.adp.assign((size_t)(lmax + 2) * S.w, 0.0);
  const double xc = S.ct;
  auto AP = [&](int l, int mm) -> double & { return S.ap[(size_t)l * S.w + mm]; };
  AP(0, 0) = 1.0;
  const double somx2 = std::sqrt((1.0 - xc) * (1.0 + xc));
  double fact = 1.0;
  for (int mm = 1; mm <= mmax; ++mm) {
    AP(mm, mm) = AP(mm - 1, mm - 1) * fact * somx2;
    fact = fact + 2.0;
  }
  for (int mm = 0; mm <= mmax; ++mm) AP(mm + 1, mm) = xc * (2 * mm + 1) * AP(mm, mm);
  for (int l = 2; l <= lmax; ++l)
    for (int mm = 0; mm <= l - 2; ++mm)
      AP(l, mm) = (xc * (2.0 * l - 1) * AP(l - 1, mm) - (l + mm - 1) * AP(l - 2, mm)) / (l - mm);
  // dalpol2
  auto ADP = [&](int l, int mm) -> double & { return S.adp[(size_t)l * S.w + mm]; };
  if (xc == 1.0 || xc == -1.0) {
    for (int l = 0; l <= lmax; ++l) {
      ADP(l, 0) = 0.0;
      if (xc == 1.0) ADP(l, 0) = l * (l + 1.0) * 0.5;
      if (xc == -1.0) ADP(l, 0) = std::pow(-1.0, l + 1) * l * (l + 1.0) * 0.5;
      for (int mm = 1; mm <= mmax; ++mm) ADP(l, mm) = 0.0;
    }
  } else {
    for (int l = 0; l <= lmax; ++l)
      for (int mm = 0; mm <= mmax; ++mm) {
        const double f = 1.0 / std::sqrt(1.0 - xc * xc);
        ADP(l, mm) = f * (AP(l, mm + 1) - f * mm * xc * AP(l, mm));
      }
  }
  return S;
}

// one basis value: norm * r^l * {1, cos m phi, sin m phi} * P_l^|m|
double sphe_value(const Mmij &m, const LegSphe &S, int ii) {
  const int l = m.lstpl[ii], mm = m.lstpm[ii];
  if (mm == 0) return S.ar[l] * S.P(l, 0);
  if (mm > 0) return S.ar[l] * S.ac[mm] * S.P(l, mm);
  return S.ar[l] * S.as[-mm] * S.P(l, -mm);
}

}  // namespace

// rect_rf1.f90 / sphe_rf1.f90 -> s.egsbpb (and the forces)
void mmij_energy(State &s, bool qforces) {
  const Mmij &m = s.mm;
  const int nt = m.ntpol;
  std::vector<double> coef(nt, 0.0), mq(nt, 0.0);
  const int i0 = s.nsites + s.nfix + 1;
  std::vector<LegRect> LR(s.ntot + 1);
  std::vector<LegSphe> LS(s.ntot + 1);
  std::vector<char> inr(s.ntot + 1, 0);
  const double srdist2 = m.srdist * m.srdist;
  double ist_last = 0.0;
  for (int i = i0; i <= s.ntot; ++i) {
    const double charge = s.cg[std::abs(s.typei[i])];
    const double xg = s.x[i], yg = s.y[i], zg = s.z[i];
    if (m.rect) {
      if (!in_rect(m, xg, yg, zg)) continue;
      inr[i] = 1;
      LR[i] = legendre_rect(m, xg, yg, zg);
      for (int ii = 0; ii < nt; ++ii)
        coef[ii] = coef[ii] + charge * m.bnorm[ii] * LR[i].lx[m.lstpx[ii]] *
                                  LR[i].ly[m.lstpy[ii]] * LR[i].lz[m.lstpz[ii]];
    } else {
      if (!(xg * xg + yg * yg + zg * zg <= srdist2)) continue;
      inr[i] = 1;
      LS[i] = legendre_sphe(m, xg, yg, zg, 10.0);  // sphe_rf1.f90:46 ist=10/st
      ist_last = LS[i].ist;
      for (int ii = 0; ii < nt; ++ii) {
        const int l = m.lstpl[ii], mm = m.lstpm[ii];
        const double norm = m.bnorm[ii];
        const LegSphe &S = LS[i];
        if (l >= 0 && mm == 0)
          coef[ii] = coef[ii] + charge * norm * S.ar[l] * S.P(l, 0);
        else if (l > 0 && mm > 0)
          coef[ii] = coef[ii] + charge * norm * S.ar[l] * S.ac[mm] * S.P(l, mm);
        else if (l > 0 && mm < 0)
          coef[ii] = coef[ii] + charge * norm * S.ar[l] * S.as[-mm] * S.P(l, -mm);
      }
    }
  }
  for (int ii = 0; ii < nt; ++ii) {
    mq[ii] = 0.0;
    for (int jj = 0; jj < nt; ++jj)
      mq[ii] = m.rect ? mq[ii] + m.mmij[(size_t)ii * nt + jj] * coef[jj] * m.rfscal
                      : mq[ii] + m.mmij[(size_t)ii * nt + jj] * coef[jj];
  }
  double e = 0.0;
  for (int ii = 0; ii < nt; ++ii) e = e + 0.5 * coef[ii] * mq[ii];
  s.egsbpb = e * s.celec;
  if (!qforces) return;
  for (int i = i0; i <= s.ntot; ++i) {
    if (!inr[i]) continue;
    const double ccc = s.cg[std::abs(s.typei[i])] * s.celec;
    double fxr = 0.0, fyr = 0.0, fzr = 0.0;
    if (m.rect) {
      const LegRect &L = LR[i];
      const double xs[3] = {m.xscal * s.x[i], m.yscal * s.y[i], m.zscal * s.z[i]};
      const int np[3] = {m.xnpol, m.ynpol, m.znpol};
      const double sc[3] = {m.xscal, m.yscal, m.zscal};
      const std::vector<double> *lp[3] = {&L.lx, &L.ly, &L.lz};
      std::vector<double> d[3];
      for (int a = 0; a < 3; ++a) {  // rect_rf1.f90:88-118
        d[a].assign(std::max(np[a], 3), 0.0);
        d[a][0] = 0.0;
        d[a][1] = 1.0;
        d[a][2] = 3.0 * xs[a];
        for (int n = 3; n <= np[a] - 1; ++n) d[a][n] = xs[a] * d[a][n - 1] + n * (*lp[a])[n - 1];
        for (int n = 0; n < np[a]; ++n) d[a][n] = d[a][n] * sc[a];
      }
      for (int ii = 0; ii < nt; ++ii) {
        const double norm = m.bnorm[ii];
        const double xl = L.lx[m.lstpx[ii]], yl = L.ly[m.lstpy[ii]], zl = L.lz[m.lstpz[ii]];
        const double dx = norm * d[0][m.lstpx[ii]] * yl * zl;
        const double dy = norm * xl * d[1][m.lstpy[ii]] * zl;
        const double dz = norm * xl * yl * d[2][m.lstpz[ii]];
        fxr = fxr - dx * mq[ii];
        fyr = fyr - dy * mq[ii];
        fzr = fzr - dz * mq[ii];
      }
    } else {
      const LegSphe &S = LS[i];
      const double ist = ist_last;  // sphe_rf1.f90:128-150: the last ion's value
      for (int ii = 0; ii < nt; ++ii) {
        const int l = m.lstpl[ii];
        int mm = m.lstpm[ii];
        const double norm = m.bnorm[ii];
        double dr = 0, ddt = 0, dp = 0;
        if (mm == 0) {
          if (l != 0) {
            const double rpl = S.ar[l - 1];
            dr = l * rpl * S.P(l, 0);
            ddt = -rpl * S.dP(l, 0) * S.st;
          }
        } else if (mm > 0) {
          const double rpl = S.ar[l - 1], cmp = S.ac[mm], apl = S.P(l, mm);
          dr = l * rpl * cmp * apl;
          ddt = -rpl * cmp * S.dP(l, mm) * S.st;
          dp = -rpl * mm * S.as[mm] * apl * ist;
          if (S.st == 0.0) dp = 0.0;
        } else {
          mm = -mm;
          const double rpl = S.ar[l - 1], smp = S.as[mm], apl = S.P(l, mm);
          dr = l * rpl * smp * apl;
          ddt = -rpl * smp * S.dP(l, mm) * S.st;
          dp = rpl * mm * S.ac[mm] * apl * ist;
          if (S.st == 0.0) dp = 0.0;
        }
        const double dx = norm * (dr * S.st * S.cp + ddt * S.ct * S.cp - dp * S.sp);
        const double dy = norm * (dr * S.st * S.sp + ddt * S.ct * S.sp + dp * S.cp);
        const double dz = norm * (dr * S.ct - ddt * S.st);
        fxr = fxr - dx * mq[ii];
        fyr = fyr - dy * mq[ii];
        fzr = fzr - dz * mq[ii];
      }
    }
    s.fx[i] = s.fx[i] + fxr * ccc;
    s.fy[i] = s.fy[i] + fyr * ccc;
    s.fz[i] = s.fz[i] + fzr * ccc;
  }
}

// rect_rf0.f90 / sphe_rf0.f90: the reaction-field energy of particle j,
// E(coef) - E(coef without j), with j at (xj, yj, zj); 0 when j is not a
// mobile ion or lies outside the region
double mmij_interact(const State &s, double xj, double yj, double zj, int j, int jtype) {
  const Mmij &m = s.mm;
  const int nt = m.ntpol;
  const int i0 = s.nsites + s.nfix + 1;
  const int last = j == s.ntot + 1 ? s.ntot + 1 : s.ntot;
  std::vector<double> coef(nt, 0.0), coef2(nt, 0.0), bj(nt, 0.0);
  const double srdist2 = m.srdist * m.srdist;
  bool jin = false;
  for (int i = i0; i <= last; ++i) {
    int itype;
    double xg, yg, zg;
    if (i == j) {
      itype = jtype;
      xg = xj;
      yg = yj;
      zg = zj;
    } else {
      itype = std::abs(s.typei[i]);
      xg = s.x[i];
      yg = s.y[i];
      zg = s.z[i];
    }
    const double charge = s.cg[itype];
    std::vector<double> b(nt, 0.0);
    if (m.rect) {
      if (!in_rect(m, xg, yg, zg)) continue;
      const LegRect L = legendre_rect(m, xg, yg, zg);
      for (int ii = 0; ii < nt; ++ii)
        b[ii] = m.bnorm[ii] * L.lx[m.lstpx[ii]] * L.ly[m.lstpy[ii]] * L.lz[m.lstpz[ii]];
    } else {
      if (!(xg * xg + yg * yg + zg * zg <= srdist2)) continue;
      const LegSphe S = legendre_sphe(m, xg, yg, zg, 1.0);  // sphe_rf0: ist = 1/st
      for (int ii = 0; ii < nt; ++ii) b[ii] = m.bnorm[ii] * sphe_value(m, S, ii);
    }
    for (int ii = 0; ii < nt; ++ii) coef[ii] = coef[ii] + charge * b[ii];
    if (i == j) {
      jin = true;
      bj = b;
    }
  }
  if (!jin) return 0.0;
  const double charge = s.cg[jtype];
  for (int ii = 0; ii < nt; ++ii) coef2[ii] = coef[ii] - charge * bj[ii];
  double e = 0.0;
  for (int ii = 0; ii < nt; ++ii) {
    const double ci = coef[ii], cj = coef2[ii];
    e = e + 0.5 * (ci * ci - cj * cj) * m.mmij[(size_t)ii * nt + ii];
    for (int jj = ii + 1; jj < nt; ++jj)
      e = e + (ci * coef[jj] - cj * coef2[jj]) * m.mmij[(size_t)ii * nt + jj];
  }
  return m.rect ? e * s.celec * m.rfscal : e * s.celec;
}

}  // namespace bref
