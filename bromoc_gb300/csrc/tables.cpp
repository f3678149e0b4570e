// Effective-potential table construction (setup, host side).
//
// The reference turns a knot table (r_k, U_k) into quadratic pieces
// U(r) = p1 + r (p2 + r p3), one per knot, through five linear passes
// (polynom.f90:20-169): averaged local parabolas, derivative continuity at the
// knots, piecewise-linear interpolation of those derivatives, integration
// back to parabolas anchored at U_1, and a correction restoring U_n.  The
// result is linear in the knot values, which the adjoint relies on.  The core
// (a/r^12 + b below the first knot) and the tail (a/r^6 + Coulomb beyond the
// last) are fitted to the end knots (splinepot.f90:28-84).
#include <cmath>
#include <vector>

#include "../../include/bromoc_gpu.h"

namespace {

struct Piece {
  double c0, c1, c2;  // U = c0 + r (c1 + r c2)
};

double eval(const Piece &q, double r) { return q.c0 + r * (q.c1 + r * q.c2); }

// Quadratic pieces with end derivatives d_first, d_last and the last piece's
// second-derivative slope dd_last.
std::vector<Piece> quad_table(const double *r, const double *u, int n,
                              double d_first, double d_last, double dd_last) {
  std::vector<Piece> q(n);
  if (n == 1) {
    q[0] = {u[0], 0.0, 0.0};
    return q;
  }
  if (n == 2) {
    const double s = (u[1] - u[0]) / (r[1] - r[0]);
    q[0] = q[1] = {u[0] - s * r[0], s, 0.0};
    return q;
  }
  // pass 1: parabola through three neighbours, averaged with the previous
  // one; the first and last honour the given end derivatives.
  auto through3 = [&](int k) {
    const double s_r = (u[k + 1] - u[k]) / (r[k + 1] - r[k]);
    const double s_l = (u[k] - u[k - 1]) / (r[k] - r[k - 1]);
    Piece p;
    p.c2 = (s_r - s_l) / (r[k + 1] - r[k - 1]);
    p.c1 = s_r - p.c2 * (r[k + 1] + r[k]);
    p.c0 = u[k] - r[k] * (p.c1 + p.c2 * r[k]);
    return p;
  };
  auto average_into = [](Piece &a, const Piece &b) {
    a.c2 = 0.5 * (a.c2 + b.c2);
    a.c1 = 0.5 * (a.c1 + b.c1);
    a.c0 = 0.5 * (a.c0 + b.c0);
  };
  {
    const double h = 1.0 / (r[1] - r[0]);
    Piece &p = q[0];
    p.c2 = ((u[1] - u[0]) * h - d_first) * h;
    p.c1 = d_first - 2.0 * p.c2 * r[0];
    p.c0 = u[0] - r[0] * (p.c1 + p.c2 * r[0]);
  }
  q[1] = through3(1);
  for (int k = 2; k <= n - 2; ++k) {
    q[k] = through3(k);
    average_into(q[k - 1], q[k]);
  }
  {
    const double h = 1.0 / (r[n - 1] - r[n - 2]);
    Piece &p = q[n - 1];
    p.c2 = (d_last - (u[n - 1] - u[n - 2]) * h) * h;
    p.c1 = d_last - 2.0 * p.c2 * r[n - 1];
    p.c0 = u[n - 1] - r[n - 1] * (p.c1 + p.c2 * r[n - 1]);
    average_into(q[n - 2], p);
  }
  // pass 2: knot derivatives, mean of the two pieces meeting at a knot
  std::vector<double> dk(n);
  dk[0] = q[0].c1 + 2.0 * q[0].c2 * r[0];
  for (int k = 1; k <= n - 2; ++k)
    dk[k] = 0.5 * (q[k].c1 + 2.0 * q[k].c2 * r[k] + q[k - 1].c1 +
                   2.0 * q[k - 1].c2 * r[k]);
  dk[n - 1] = q[n - 1].c1 + 2.0 * q[n - 1].c2 * r[n - 1];
  // pass 3: derivative as a line per interval (slope g, intercept a)
  std::vector<double> a(n), g(n);
  for (int k = 0; k <= n - 2; ++k) {
    const double h = 1.0 / (r[k + 1] - r[k]);
    g[k] = (dk[k + 1] - dk[k]) * h;
    a[k] = (dk[k] * r[k + 1] - dk[k + 1] * r[k]) * h;
  }
  g[n - 1] = dd_last;
  a[n - 1] = dk[n - 1] - dd_last * r[n - 1];
  // pass 4: integrate, continuous at every knot, anchored at u[0]
  q[0].c2 = 0.5 * g[0];
  q[0].c1 = a[0];
  q[0].c0 = u[0] - r[0] * (q[0].c1 + q[0].c2 * r[0]);
  for (int k = 1; k < n; ++k) {
    const Piece prev = q[k - 1];
    q[k].c2 = 0.5 * g[k];
    q[k].c1 = a[k];
    q[k].c0 = prev.c0 + r[k] * (prev.c1 - q[k].c1 + r[k] * (prev.c2 - q[k].c2));
  }
  // pass 5: restore the last value with a correction that keeps the end
  // derivatives; the curvature term uses the reference's nominal knot grid
  // r_0 + h (k) with h = (r_1 - r_0)/(n-1)  (polynom.f90:104-111)
  const double un = eval(q[n - 1], r[n - 1]);
  const double b = 2.0 * (u[n - 1] - un) / (r[n - 1] - r[0]);
  const double c = -b * r[0] * 0.5;
  const double h = (r[1] - r[0]) / (n - 1);
  for (int k = 0; k < n - 1; ++k) {
    q[k].c0 += c;
    q[k].c1 += b;
    q[k].c2 += -b * 0.5 / (r[k] + h * k);
  }
  q[n - 1].c0 += c;
  q[n - 1].c1 += b;
  q[n - 1].c2 += -b * 0.5 / r[n - 1];
  return q;
}

}  // namespace

extern "C" int bromoc_gpu_efpot_from_knots(int32_t n, const double *xx,
                                           const double *yy, double fct,
                                           int32_t qchr, double *ep,
                                           double *sc3, double *dm2o,
                                           double *dmio) {
  if (n < 3 || !xx || !yy || !ep || !sc3 || !dm2o || !dmio) return BROMOC_E_ARG;
  const double r0 = xx[0], r1 = xx[1], rn = xx[n - 1];
  if (r0 == 0.0 || rn == 0.0) return BROMOC_E_ARG;  // division by zero upstream
  const double kf = qchr ? fct : 0.0;
  *dmio = r0;
  dm2o[0] = r0 * r0;
  dm2o[1] = rn * rn;
  // tail a/r^6 (+ Coulomb kf/r) through the last knot; its slope and
  // curvature close the table
  const double rn5 = std::pow(rn, 5);
  sc3[2] = (rn * yy[n - 1] - kf) * rn5;
  const double d_last = -kf / (rn * rn) - 6.0 * sc3[2] / std::pow(rn, 7);
  const double dd_last = 2.0 * kf / std::pow(rn, 3) + 42.0 * sc3[2] / std::pow(rn, 8);
  // core a/r^12 + b through the first two knots
  const double p0 = std::pow(r0, 12), p1 = std::pow(r1, 12);
  const double inv = 1.0 / (p0 - p1);
  sc3[0] = (yy[1] - yy[0]) * p1 * p0 * inv;
  sc3[1] = (yy[0] * p0 - yy[1] * p1) * inv;
  const double d_first = -12.0 * sc3[0] / std::pow(r0, 13);
  const std::vector<Piece> q = quad_table(xx, yy, n, d_first, d_last, dd_last);
  for (int k = 0; k < n; ++k) {
    ep[3 * k + 0] = q[k].c0;
    ep[3 * k + 1] = q[k].c1;
    ep[3 * k + 2] = q[k].c2;
  }
  return BROMOC_OK;
}
