// ORACLE -- test infrastructure only.  DNA bonded and Go-like terms between
// interaction sites, restated from the reference in its expression order:
//   ENERGY    energy.mono.f90:196-582 (bonds, angles, torsions; stacking,
//             base pairs, excluded volume, P-P electrostatics, solvent
//             term; APFOR; CONTRANS)
//   INTERACT  interact.f90:211-334 (the terms that involve site j, at the
//             stored positions; angbond.f90, angdih.f90)
// Lists as built by bonds.f90, angles.f90, dihedral.f90 and go_qq.f90,
// passed in through bromoc_ref_set_nucleotides.
#include <cmath>

#include "ref_state.h"

namespace bref {

// grandmod.f90:74-98
bool outbox(const State &s, double xi, double yi, double zi) {
  const bromoc_system &y = s.sys;
  if (y.shape == BROMOC_SPHERE)
    return (xi - y.cx) * (xi - y.cx) + (yi - y.cy) * (yi - y.cy) + (zi - y.cz) * (zi - y.cz) >
           s.rsphe2;
  if (y.shape == BROMOC_ECYL) {
    const double u = (xi - y.cx) * s.iecx, v = (yi - y.cy) * s.iecy;
    return u * u + v * v > 1.0 || zi < s.lz2m || zi > s.lz2p;
  }
  return xi < s.lx2m || xi > s.lx2p || yi < s.ly2m || yi > s.ly2p || zi < s.lz2m ||
         zi > s.lz2p;
}

static void cross_product(const double u[3], const double v[3], double w[3]) {
  w[0] = u[1] * v[2] - u[2] * v[1];
  w[1] = u[2] * v[0] - u[0] * v[2];
  w[2] = u[0] * v[1] - u[1] * v[0];
}

static double dot(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// angbond.f90: vecR columns r1 = x1 - x2, r2 = x3 - x2
static double angbond(const double r1[3], const double r2[3]) {
  double R1 = std::sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
  double R2 = std::sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
  double prod = 0.0;
  for (int i = 0; i < 3; ++i) prod = prod + r1[i] * r2[i];
  return std::acos(prod / (R1 * R2));
}

// angdih.f90: vecR columns r1 = x2 - x1, r2 = x3 - x2, r3 = x4 - x3
static double angdih(const double r1[3], const double r2[3], const double r3[3]) {
  double n1[3], n2[3];
  n1[0] = r1[1] * r2[2] - r1[2] * r2[1];
  n1[1] = r1[2] * r2[0] - r1[0] * r2[2];
  n1[2] = r1[0] * r2[1] - r1[1] * r2[0];
  n2[0] = r2[1] * r3[2] - r2[2] * r3[1];
  n2[1] = r2[2] * r3[0] - r2[0] * r3[2];
  n2[2] = r2[0] * r3[1] - r2[1] * r3[0];
  const double R2 = std::sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
  double sinphi = 0.0, cosphi = 0.0;
  for (int i = 0; i < 3; ++i) {
    sinphi = sinphi + r1[i] * n2[i];
    cosphi = cosphi + n1[i] * n2[i];
  }
  sinphi = R2 * sinphi;
  return std::atan2(sinphi, cosphi);
}

namespace {

struct Acc {  // fx(isite) = fx(isite) + f for free sites
  State &s;
  void add(int i, const double f[3], double sign) {
    if (!s.stfree[i]) return;
    s.fx[i] += sign * f[0];
    s.fy[i] += sign * f[1];
    s.fz[i] += sign * f[2];
  }
};

void sep(const State &s, int a, int b, double v[3]) {  // v = r_b - r_a
  v[0] = s.x[b] - s.x[a];
  v[1] = s.y[b] - s.y[a];
  v[2] = s.z[b] - s.z[a];
}

}  // namespace

// energy.mono.f90:196-582
void nucl_energy(State &s, uint32_t mask, bool qforces) {
  const Nucl &n = s.nuc;
  s.ebond = s.eang = s.edihe = s.estack = s.ebp = s.eex = s.eqq = s.esolv = s.econ = 0.0;
  if (!n.on || !s.qnucl()) return;
  const double eps = n.epsnuc;
  Acc acc{s};
  auto ok2 = [&](int a, int b) { return (qforces && s.stfree[a]) || s.stfree[b]; };
  if (mask & BROMOC_M_BOND) {
    for (size_t k = 0; k < n.distbond.size(); ++k) {  // :205-230
      const int i1 = n.bond[2 * k], i2 = n.bond[2 * k + 1];
      const double dd = n.distbond[k];
      double v1[3];
      sep(s, i1, i2, v1);
      const double dist = std::sqrt(dot(v1, v1));
      const double vard = dist - dd;
      const double vard2 = vard * vard;
      s.ebond = s.ebond + eps * vard2 * (1.0 + 100.0 * vard2);
      if (ok2(i1, i2)) {
        const double de = eps * vard * (2.0 + 400.0 * vard2) / dist;
        const double f1[3] = {de * v1[0], de * v1[1], de * v1[2]};
        acc.add(i1, f1, 1.0);
        acc.add(i2, f1, -1.0);
      }
    }
    for (size_t k = 0; k < n.valangle.size(); ++k) {  // :234-276
      const int i1 = n.angle[3 * k], i2 = n.angle[3 * k + 1], i3 = n.angle[3 * k + 2];
      const double ang0 = n.valangle[k];
      double v1[3], v2[3];
      sep(s, i2, i1, v1);
      sep(s, i2, i3, v2);
      const double m1 = dot(v1, v1), m2 = dot(v2, v2), m3 = dot(v1, v2);
      const double modval = 1.0 / std::sqrt(m1 * m2);
      const double ang = std::acos(m3 * modval);
      const double varang = ang - ang0;
      s.eang = s.eang + 700.0 * eps * (varang * varang);
      if ((qforces && s.stfree[i1]) || s.stfree[i2] || s.stfree[i3]) {
        const double de = 1400.0 * eps * varang * modval / std::sin(ang);
        const double f1[3] = {de * v1[0], de * v1[1], de * v1[2]};
        const double f2[3] = {de * v2[0], de * v2[1], de * v2[2]};
        const double f12[3] = {f1[0] + f2[0], f1[1] + f2[1], f1[2] + f2[2]};
        acc.add(i1, f2, 1.0);
        acc.add(i2, f12, -1.0);
        acc.add(i3, f1, 1.0);
      }
    }
    for (size_t k = 0; k < n.valdihe.size(); ++k) {  // :279-336
      const int i1 = n.dihe[4 * k], i2 = n.dihe[4 * k + 1], i3 = n.dihe[4 * k + 2],
                i4 = n.dihe[4 * k + 3];
      const double dihe0 = n.valdihe[k];
      double v1[3], v2[3], v3[3], n1[3], n2[3];
      sep(s, i2, i1, v1);
      sep(s, i2, i3, v2);
      sep(s, i4, i3, v3);
      cross_product(v1, v2, n1);
      cross_product(v2, v3, n2);
      const double v22 = dot(v2, v2);
      const double v2v = std::sqrt(v22);
      const double av = dot(v1, n2);
      const double bv = dot(n1, n2);
      const double dihe = std::atan2(v2v * av, bv);
      const double vardihe = dihe - dihe0;
      s.edihe = s.edihe + 28.0 * eps * (1.0 - std::cos(vardihe));
      if ((qforces && s.stfree[i1]) || s.stfree[i2] || s.stfree[i3] || s.stfree[i4]) {
        const double n1v = dot(n1, n1), n2v = dot(n2, n2);
        double v12 = dot(v1, v2), v23 = dot(v2, v3);
        const double de = 28.0 * eps * std::sin(vardihe) * v2v;
        double f1[3], f2[3], f3[3], f4[3];
        for (int m = 0; m < 3; ++m) {
          f1[m] = -de / n1v * n1[m];
          f4[m] = de / n2v * n2[m];
        }
        const double iv22 = 1.0 / v22;
        v12 = v12 * iv22;
        v23 = v23 * iv22;
        for (int m = 0; m < 3; ++m) {
          f2[m] = -f1[m] + v12 * f1[m] - v23 * f4[m];
          f3[m] = -f4[m] - v12 * f1[m] + v23 * f4[m];
        }
        acc.add(i1, f1, 1.0);
        acc.add(i2, f2, 1.0);
        acc.add(i3, f3, 1.0);
        acc.add(i4, f4, 1.0);
      }
    }
  }
  if (mask & BROMOC_M_NONBOND) {
    // pair terms: F on i1 is -de v1, on i2 +de v1 with v1 = r2 - r1
    auto pair_force = [&](int i1, int i2, double de, const double v1[3]) {
      if (!ok2(i1, i2)) return;
      const double f1[3] = {de * v1[0], de * v1[1], de * v1[2]};
      acc.add(i1, f1, -1.0);
      acc.add(i2, f1, 1.0);
    };
    for (size_t k = 0; k < n.sgstack.size(); ++k) {  // :341-366
      const int i1 = n.stack[2 * k], i2 = n.stack[2 * k + 1];
      double v1[3];
      sep(s, i1, i2, v1);
      const double dist2 = dot(v1, v1);
      const double idist2 = 1.0 / dist2;
      const double cte1 = pow3(n.sgstack[k] * n.sgstack[k] * idist2);
      s.estack = s.estack + 4.0 * eps * cte1 * (cte1 - 1.0);
      pair_force(i1, i2, 24.0 * eps * cte1 * (2.0 * cte1 - 1.0) * idist2, v1);
    }
    for (size_t k = 0; k < n.sgbp.size(); ++k) {  // :368-397
      const int i1 = n.bp[2 * k], i2 = n.bp[2 * k + 1];
      const double epsln =
          n.bpgc[k] ? 2.532 * eps * n.scalepairing : 2.0 * eps * n.scalepairing;
      double v1[3];
      sep(s, i1, i2, v1);
      const double dist2 = dot(v1, v1);
      const double idist2 = 1.0 / dist2;
      const double cte1 = n.sgbp[k] * n.sgbp[k] * idist2;
      const double c5 = cte1 * cte1 * cte1 * cte1 * cte1;
      s.ebp = s.ebp + epsln * c5 * (20.0 * cte1 - 24.0);
      pair_force(i1, i2, 240.0 * epsln * c5 * (cte1 - 1.0) * idist2, v1);
    }
    for (size_t k = 0; k < n.sgex.size(); ++k) {  // :399-426
      const int i1 = n.ex[2 * k], i2 = n.ex[2 * k + 1];
      double v1[3];
      sep(s, i1, i2, v1);
      const double dist2 = dot(v1, v1);
      const double idist2 = 1.0 / dist2;
      const double sgex2 = n.sgex[k] * n.sgex[k];
      if (dist2 < sgex2) {
        const double cte1 = pow3(sgex2 * idist2);
        s.eex = s.eex + 4.0 * eps * cte1 * (cte1 - 1.0) + eps;
        pair_force(i1, i2, 24.0 * eps * cte1 * (2.0 * cte1 - 1.0) * idist2, v1);
      }
    }
    for (size_t k = 0; k < n.qq.size() / 2; ++k) {  // :428-479
      const int i1 = n.qq[2 * k], i2 = n.qq[2 * k + 1];
      double v1[3];
      sep(s, i1, i2, v1);
      const double dist = std::sqrt(dot(v1, v1));
      const double idist = 1.0 / dist;
      bool deby = n.qdeby == 1;
      if (n.qdeby == 2)
        deby = outbox(s, s.x[i1], s.y[i1], s.z[i1]) && outbox(s, s.x[i2], s.y[i2], s.z[i2]);
      if (deby) {
        const double idistkd = std::exp(-dist * n.ikappa);
        s.eqq = s.eqq + n.fctn * idist * idistkd;
        pair_force(i1, i2, n.fctn * (dist + n.kappa) * pow3(idist) * n.ikappa * idistkd, v1);
      } else {
        s.eqq = s.eqq + n.fctn * idist;
        pair_force(i1, i2, n.fctn * pow3(idist), v1);
      }
    }
    if (n.qsolv)
      for (size_t k = 0; k < n.slv.size() / 2; ++k) {  // :481-503
        const int i1 = n.slv[2 * k], i2 = n.slv[2 * k + 1];
        double v1[3];
        sep(s, i1, i2, v1);
        const double dist = std::sqrt(dot(v1, v1));
        const double cte1 = std::exp((13.38 - dist) * 0.1875);
        s.esolv = s.esolv + n.epsolv * ((1.0 - cte1) * (1.0 - cte1)) - n.epsolv;
        pair_force(i1, i2, 0.375 * n.epsolv * cte1 * (cte1 - 1.0) / dist, v1);
      }
  }
  // APFOR :506-515
  for (size_t k = 0; k < n.sn.size(); ++k) {
    const int j = n.sn[k];
    if (qforces && s.stfree[j]) {
      s.fx[j] += n.af[3 * k];
      s.fy[j] += n.af[3 * k + 1];
      s.fz[j] += n.af[3 * k + 2];
    }
  }
  // CONTRANS :516-581 (x, y and z alike)
  const int ctn = (int)n.csn.size();
  const double insites = 1.0 / s.nsites;
  const int n1st = n.nsites1st;
  std::vector<double> *pos[3] = {&s.x, &s.y, &s.z};
  std::vector<double> *frc[3] = {&s.fx, &s.fy, &s.fz};
  const std::vector<double> *kk[3] = {&n.kx, &n.ky, &n.kz};
  const std::vector<double> *cc[3] = {&n.contrx, &n.contry, &n.contrz};
  for (int i = 0; i < ctn; ++i) {
    const int j = n.csn[i];
    for (int a = 0; a < 3; ++a) {
      const double kv = (*kk[a])[i];
      if (kv == 0.0) continue;
      std::vector<double> &p = *pos[a], &f = *frc[a];
      const std::vector<double> &c = *cc[a];
      if (j == 0) {
        if (n.qunsplit) {
          double sm = 0.0;
          for (int m = 1; m <= n1st; ++m) sm = sm + p[m];
          double con = sm * insites * 2.0 - c[i];
          for (int m = 1; m <= n1st; ++m) f[m] = f[m] - kv * con * insites * 2.0;
          s.econ = s.econ + 0.5 * kv * (con * con);
          sm = 0.0;
          for (int m = 1 + n1st; m <= s.nsites; ++m) sm = sm + p[m];
          con = sm * insites * 2.0 - c[ctn];
          for (int m = 1 + n1st; m <= s.nsites; ++m) f[m] = f[m] - kv * con * insites * 2.0;
          s.econ = s.econ + 0.5 * kv * (con * con);
        } else {
          double sm = 0.0;
          for (int m = 1; m <= s.nsites; ++m) sm = sm + p[m];
          const double con = sm * insites - c[i];
          for (int m = 1; m <= s.nsites; ++m) f[m] = f[m] - kv * con * insites;
          s.econ = s.econ + 0.5 * kv * (con * con);
        }
      } else {
        f[j] = f[j] - kv * (p[j] - c[i]);
        s.econ = s.econ + 0.5 * kv * ((p[j] - c[i]) * (p[j] - c[i]));
      }
    }
  }
}

// interact.f90:211-334: terms of site j at the stored positions
void nucl_interact(const State &s, uint32_t mask, int j, double &dener) {
  const Nucl &n = s.nuc;
  if (!n.on) return;
  const double eps = n.epsnuc;
  auto d2of = [&](int a, int b) {
    return (s.x[b] - s.x[a]) * (s.x[b] - s.x[a]) + (s.y[b] - s.y[a]) * (s.y[b] - s.y[a]) +
           (s.z[b] - s.z[a]) * (s.z[b] - s.z[a]);
  };
  if (mask & BROMOC_M_BOND) {
    for (size_t k = 0; k < n.distbond.size(); ++k) {
      const int i1 = n.bond[2 * k], i2 = n.bond[2 * k + 1];
      if (i1 != j && i2 != j) continue;
      const double dist = std::sqrt((s.x[i1] - s.x[i2]) * (s.x[i1] - s.x[i2]) +
                                    (s.y[i1] - s.y[i2]) * (s.y[i1] - s.y[i2]) +
                                    (s.z[i1] - s.z[i2]) * (s.z[i1] - s.z[i2]));
      const double vard = dist - n.distbond[k];
      dener = dener + eps * (vard * vard) * (1.0 + 100.0 * (vard * vard));
    }
    for (size_t k = 0; k < n.valangle.size(); ++k) {
      const int i1 = n.angle[3 * k], i2 = n.angle[3 * k + 1], i3 = n.angle[3 * k + 2];
      if (i1 != j && i2 != j && i3 != j) continue;
      const double r1[3] = {s.x[i1] - s.x[i2], s.y[i1] - s.y[i2], s.z[i1] - s.z[i2]};
      const double r2[3] = {s.x[i3] - s.x[i2], s.y[i3] - s.y[i2], s.z[i3] - s.z[i2]};
      const double varang = angbond(r1, r2) - n.valangle[k];
      dener = dener + 700.0 * eps * (varang * varang);
    }
    for (size_t k = 0; k < n.valdihe.size(); ++k) {
      const int i1 = n.dihe[4 * k], i2 = n.dihe[4 * k + 1], i3 = n.dihe[4 * k + 2],
                i4 = n.dihe[4 * k + 3];
      if (i1 != j && i2 != j && i3 != j && i4 != j) continue;
      const double r1[3] = {s.x[i2] - s.x[i1], s.y[i2] - s.y[i1], s.z[i2] - s.z[i1]};
      const double r2[3] = {s.x[i3] - s.x[i2], s.y[i3] - s.y[i2], s.z[i3] - s.z[i2]};
      const double r3[3] = {s.x[i4] - s.x[i3], s.y[i4] - s.y[i3], s.z[i4] - s.z[i3]};
      const double vardihe = angdih(r1, r2, r3) - n.valdihe[k];
      dener = dener + 28.0 * eps * (1.0 - std::cos(vardihe));
    }
  }
  if (mask & BROMOC_M_NONBOND) {
    for (size_t k = 0; k < n.sgstack.size(); ++k) {
      const int i1 = n.stack[2 * k], i2 = n.stack[2 * k + 1];
      if (i1 != j && i2 != j) continue;
      const double cte1 = pow3(n.sgstack[k] * n.sgstack[k] / d2of(i1, i2));
      dener = dener + 4.0 * eps * cte1 * (cte1 - 1.0);
    }
    for (size_t k = 0; k < n.sgbp.size(); ++k) {
      const int i1 = n.bp[2 * k], i2 = n.bp[2 * k + 1];
      if (i1 != j && i2 != j) continue;
      const double epsln = n.bpgc[k] ? 2.532 * eps : 2.0 * eps;
      const double cte1 = n.sgbp[k] * n.sgbp[k] / d2of(i1, i2);
      const double c5 = cte1 * cte1 * cte1 * cte1 * cte1;
      dener = dener + epsln * c5 * (20.0 * cte1 - 24.0);
    }
    for (size_t k = 0; k < n.sgex.size(); ++k) {
      const int i1 = n.ex[2 * k], i2 = n.ex[2 * k + 1];
      if (i1 != j && i2 != j) continue;
      const double dist2 = d2of(i1, i2);
      const double sgex2 = n.sgex[k] * n.sgex[k];
      if (dist2 < sgex2) {
        const double cte1 = pow3(sgex2 / dist2);
        dener = dener + 4.0 * eps * cte1 * (cte1 - 1.0) + eps;
      }
    }
    for (size_t k = 0; k < n.qq.size() / 2; ++k) {
      const int i1 = n.qq[2 * k], i2 = n.qq[2 * k + 1];
      if (i1 != j && i2 != j) continue;
      const double dist = std::sqrt(d2of(i1, i2));
      const double idist = 1.0 / dist;
      bool deby = n.qdeby == 1;
      if (n.qdeby == 2)
        deby = outbox(s, s.x[i1], s.y[i1], s.z[i1]) && outbox(s, s.x[i2], s.y[i2], s.z[i2]);
      if (!deby)
        dener = dener + n.fctn * idist;
      else
        dener = dener + n.fctn * idist * std::exp(-dist * n.ikappa);
    }
    if (n.qsolv)
      for (size_t k = 0; k < n.slv.size() / 2; ++k) {
        const int i1 = n.slv[2 * k], i2 = n.slv[2 * k + 1];
        if (i1 != j && i2 != j) continue;
        const double dist = std::sqrt(d2of(i1, i2));
        const double cte1 = std::exp((13.38 - dist) * 0.1875);
        dener = dener + n.epsolv * ((1.0 - cte1) * (1.0 - cte1)) - n.epsolv;
      }
  }
}

}  // namespace bref
