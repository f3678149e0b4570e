// ORACLE -- test infrastructure only (see ref_state.h).
// Pair laws, effective-potential tables, ENERGY driver and the noise stream.
#include <cmath>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ref_state.h"

namespace bref {

void Grid::set(const bromoc_grid &g) {
  nclx = g.nclx;
  ncly = g.ncly;
  nclz = g.nclz;
  dcel = g.dcel;
  idcel = 1.0 / dcel;
  // readphi.f90:49-51
  tranx = 0.5 * (nclx - 1) * dcel;
  trany = 0.5 * (ncly - 1) * dcel;
  tranz = 0.5 * (nclz - 1) * dcel;
  xbcen = g.xbcen;
  ybcen = g.ybcen;
  zbcen = g.zbcen;
}

void State::resize_particles(int cap) {
  capacity = cap;
  x.assign(cap + 2, 0.0);
  y.assign(cap + 2, 0.0);
  z.assign(cap + 2, 0.0);
  fx.assign(cap + 2, 0.0);
  fy.assign(cap + 2, 0.0);
  fz.assign(cap + 2, 0.0);
  typei.assign(cap + 2, 0);
  ibuffer.assign(cap + 2, 0);
  dids.assign(5 * (cap + 2), 0.0);
}

// nindex.f90:19-35
int nindex(const State &s, int itype, int jtype) {
  int maxi, mini;
  if (itype > jtype) {
    maxi = itype - s.ndna;
    mini = jtype;
  } else {
    maxi = jtype - s.ndna;
    mini = itype;
  }
  if (mini > s.ndna) return maxi * (maxi - 1) / 2 + mini - s.ndna + s.ndnaxnion;
  return (mini - 1) * s.nion + maxi;
}


// polynom.f90:172-194
void gety(const State &s, int is, double x2, double &y, double &x) {
  x = 0.0;
  if (x2 < s.dm2[2 * (is - 1) + 0]) {
    double ix2 = 1.0 / x2;
    y = s.sc[3 * (is - 1) + 0] * pow6(ix2) + s.sc[3 * (is - 1) + 1];
  } else if (x2 > s.dm2[2 * (is - 1) + 1]) {
    double ix2 = 1.0 / x2;
    if (s.qchr[is])
      y = s.sc[3 * (is - 1) + 2] * pow3(ix2) + s.fct[is] * std::sqrt(ix2);
    else
      y = s.sc[3 * (is - 1) + 2] * pow3(ix2);
  } else {
    x = std::sqrt(x2);
    int i = (int)((x - s.dmi[is]) * s.ires) + s.nxi[is];
    const double *p = &s.ep[3 * (i - 1)];
    y = p[0] + x * (p[1] + x * p[2]);
  }
}

// polynom.f90:197-230
void getyd(const State &s, int is, double x2, double &y, double &yp,
           double &x) {
  x = 0.0;
  if (x2 < s.dm2[2 * (is - 1) + 0]) {
    double ix2 = 1.0 / x2;
    double c = s.sc[3 * (is - 1) + 0] * pow6(ix2);
    y = c + s.sc[3 * (is - 1) + 1];
    yp = 12.0 * c * ix2;
  } else if (x2 > s.dm2[2 * (is - 1) + 1]) {
    double ix2 = 1.0 / x2;
    double c = s.sc[3 * (is - 1) + 2] * pow3(ix2);
    if (s.qchr[is]) {
      double f = s.fct[is] * std::sqrt(ix2);
      y = c + f;
      yp = (6.0 * c + f) * ix2;
    } else {
      y = c;
      yp = 6.0 * c * ix2;
    }
  } else {
    x = std::sqrt(x2);
    int i = (int)((x - s.dmi[is]) * s.ires) + s.nxi[is];
    const double *p = &s.ep[3 * (i - 1)];
    y = p[0] + x * (p[1] + x * p[2]);
    yp = -p[1] / x - 2.0 * p[2];
  }
}

// ---- squarespline and helpers: polynom.f90:20-169.  p(1:3,1:n) is stored
// as p[3*(i-1)+(m-1)]; 1-based helpers keep the Fortran index arithmetic.
#define P(m, i) p[3 * ((i)-1) + ((m)-1)]
#define X(i) x[(i)-1]
#define Y(i) y[(i)-1]

static void sqfit(int n, const double *x, const double *y, double *p, double d1,
                  double d2) {
  int i = 1;
  double tt = 1.0 / (X(i + 1) - X(i));
  P(3, i) = ((Y(i + 1) - Y(i)) * tt - d1) * tt;
  P(2, i) = d1 - 2.0 * P(3, i) * X(i);
  P(1, i) = Y(i) - X(i) * (P(2, i) + P(3, i) * X(i));
  i = 2;
  tt = (Y(i + 1) - Y(i)) / (X(i + 1) - X(i));
  P(3, i) = (tt - (Y(i) - Y(i - 1)) / (X(i) - X(i - 1))) / (X(i + 1) - X(i - 1));
  P(2, i) = tt - P(3, i) * (X(i + 1) + X(i));
  P(1, i) = Y(i) - X(i) * (P(2, i) + P(3, i) * X(i));
  for (i = 3; i <= n - 1; ++i) {
    tt = (Y(i + 1) - Y(i)) / (X(i + 1) - X(i));
    P(3, i) =
        (tt - (Y(i) - Y(i - 1)) / (X(i) - X(i - 1))) / (X(i + 1) - X(i - 1));
    P(2, i) = tt - P(3, i) * (X(i + 1) + X(i));
    P(1, i) = Y(i) - X(i) * (P(2, i) + P(3, i) * X(i));
    P(3, i - 1) = 0.5 * (P(3, i - 1) + P(3, i));
    P(2, i - 1) = 0.5 * (P(2, i - 1) + P(2, i));
    P(1, i - 1) = 0.5 * (P(1, i - 1) + P(1, i));
  }
  tt = 1.0 / (X(n) - X(n - 1));
  P(3, n) = (d2 - (Y(n) - Y(n - 1)) * tt) * tt;
  P(2, n) = d2 - 2.0 * P(3, n) * X(n);
  P(1, n) = Y(n) - X(n) * (P(2, n) + P(3, n) * X(n));
  P(3, n - 1) = 0.5 * (P(3, n - 1) + P(3, n));
  P(2, n - 1) = 0.5 * (P(2, n - 1) + P(2, n));
  P(1, n - 1) = 0.5 * (P(1, n - 1) + P(1, n));
}

static void fixder(int n, const double *x, const double *p, double *yp) {
  yp[0] = P(2, 1) + 2.0 * P(3, 1) * X(1);
  for (int i = 2; i <= n - 1; ++i)
    yp[i - 1] = 0.5 * (P(2, i) + 2.0 * P(3, i) * X(i) + P(2, i - 1) +
                       2.0 * P(3, i - 1) * X(i));
  yp[n - 1] = P(2, n) + 2.0 * P(3, n) * X(n);
}

// pp(1:2, 1:n) -> pp[2*(i-1)+(m-1)]
static void linipol(int n, const double *x, const double *y, double *pp,
                    double dd) {
  for (int i = 1; i <= n - 1; ++i) {
    double tt = 1.0 / (X(i + 1) - X(i));
    pp[2 * (i - 1) + 1] = (Y(i + 1) - Y(i)) * tt;
    pp[2 * (i - 1) + 0] = (Y(i) * X(i + 1) - Y(i + 1) * X(i)) * tt;
  }
  pp[2 * (n - 1) + 1] = dd;
  pp[2 * (n - 1) + 0] = Y(n) - pp[2 * (n - 1) + 1] * X(n);
}

static void intlin(int n, const double *x, const double *pp, double *p,
                   double y0) {
  P(3, 1) = pp[1] * 0.5;
  P(2, 1) = pp[0];
  P(1, 1) = y0 - X(1) * (P(2, 1) + P(3, 1) * X(1));
  for (int i = 2; i <= n; ++i) {
    P(3, i) = pp[2 * (i - 1) + 1] * 0.5;
    P(2, i) = pp[2 * (i - 1) + 0];
    P(1, i) = P(1, i - 1) +
              X(i) * (P(2, i - 1) - P(2, i) + X(i) * (P(3, i - 1) - P(3, i)));
  }
}

static void fixdy(int n, const double *x, double *p, double yn) {
  int i = 1;
  (void)(P(1, i) + X(i) * (P(2, i) + X(i) * P(3, i)));  // y0, unused upstream
  i = n;
  double ynn = P(1, i) + X(i) * (P(2, i) + X(i) * P(3, i));
  double b = 2.0 * (yn - ynn) / (X(n) - X(1));
  double c = -b * X(1) * 0.5;
  double h = (X(2) - X(1)) / (n - 1);
  for (i = 1; i <= n - 1; ++i) {
    P(1, i) = P(1, i) + c;
    P(2, i) = P(2, i) + b;
    double a = -b * 0.5 / (X(i) + h * (i - 1));
    P(3, i) = P(3, i) + a;
  }
  i = n;
  P(1, i) = P(1, i) + c;
  P(2, i) = P(2, i) + b;
  double a = -b * 0.5 / X(i);
  P(3, i) = P(3, i) + a;
}

void squarespline(int n, const double *x, const double *y, double *p,
                  double d1, double d2, double dd2) {
  if (n == 1) {
    P(3, 1) = 0.0;
    P(2, 1) = 0.0;
    P(1, 1) = Y(1);
  } else if (n == 2) {
    P(3, 1) = 0.0;
    P(2, 1) = (Y(2) - Y(1)) / (X(2) - X(1));
    P(1, 1) = Y(1) - P(2, 1) * X(1);
    P(3, 2) = P(3, 1);
    P(2, 2) = P(2, 1);
    P(1, 2) = P(1, 1);
  } else if (n > 2) {
    double y0 = Y(1), yn = Y(n);
    std::vector<double> yp(y, y + n), pp(2 * n);
    sqfit(n, x, yp.data(), p, d1, d2);
    fixder(n, x, p, yp.data());
    linipol(n, x, yp.data(), pp.data(), dd2);
    intlin(n, x, pp.data(), p, y0);
    fixdy(n, x, p, yn);
  }
}
#undef P
#undef X
#undef Y

// splinepot.f90:19-96 for one pair
void splinepot(int nn, const double *xx, const double *yy, double fct,
               bool qchr, double *p, double *sc3, double *dm2o, double *dmio) {
  *dmio = xx[0];
  dm2o[0] = xx[0] * xx[0];
  dm2o[1] = xx[nn - 1] * xx[nn - 1];
  double kf = qchr ? fct : 0.0;
  double xn = xx[nn - 1];
  sc3[2] = (xn * yy[nn - 1] - kf) * std::pow(xn, 5);
  double d2 = -kf / (xn * xn) - 6.0 * sc3[2] / std::pow(xn, 7);
  double dd2 = 2.0 * kf / std::pow(xn, 3) + 42.0 * sc3[2] / std::pow(xn, 8);
  double x1_12 = std::pow(xx[0], 12), x2_12 = std::pow(xx[1], 12);
  double dd1 = 1.0 / (x1_12 - x2_12);
  sc3[0] = (yy[1] - yy[0]) * x2_12 * x1_12 * dd1;
  sc3[1] = (yy[0] * x1_12 - yy[1] * x2_12) * dd1;
  double d1 = -12.0 * sc3[0] / std::pow(xx[0], 13);
  squarespline(nn, xx, yy, p, d1, d2, dd2);
}

// ---- noise -----------------------------------------------------------------
void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                   uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t a = (uint64_t)0xD2511F53u * c0;
    uint64_t b = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(b >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)b;
    uint32_t n2 = (uint32_t)(a >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)a;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

static inline double u01(uint32_t w) { return (double)w * 0x1p-32; }

// rgauss.f90:24: cos(rndm()*2pi)*sqrt(-2 log(rndm1())), rndm1 = 1 - rand()
static inline double box_muller(uint32_t wa, uint32_t wb) {
  return std::cos(u01(wa) * twopi) * std::sqrt(-2.0 * std::log(1.0 - u01(wb)));
}

double bd_gauss(uint64_t seed, uint64_t step, uint32_t slot, int comp) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {slot, (uint32_t)(comp >> 1), (uint32_t)step,
                     ((uint32_t)(step >> 32) & 0x00FFFFFFu) | (1u << 24)};
  uint32_t w[4];
  philox4x32_10(ctr, key, w);
  return (comp & 1) ? box_muller(w[2], w[3]) : box_muller(w[0], w[1]);
}

// The uniforms of Metropolis moves: the GCMC stream's layout under its own
// tag, so the two never share a counter.
double mc_uniform(uint64_t seed, uint64_t cycle, uint32_t move, uint32_t draw) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {move, draw >> 2, (uint32_t)cycle,
                     ((uint32_t)(cycle >> 32) & 0x00FFFFFFu) | (3u << 24)};
  uint32_t w[4];
  philox4x32_10(ctr, key, w);
  return u01(w[draw & 3]);
}

double gcmc_uniform(uint64_t seed, uint64_t cycle, uint32_t attempt,
                    uint32_t draw) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t ctr[4] = {attempt, draw >> 2, (uint32_t)cycle,
                     ((uint32_t)(cycle >> 32) & 0x00FFFFFFu) | (2u << 24)};
  uint32_t w[4];
  philox4x32_10(ctr, key, w);
  return u01(w[draw & 3]);
}

// Ion-ion pairs for mobile j in [jlo, jhi], all ions i < j, in the loop order
// of energy.mono.f90:120-192.  e = {eelec, evdw, esrpmf, eefpot}.
static void ionion_range(const State &s, int jlo, int jhi, bool qforces,
                         double *fx, double *fy, double *fz, double e[4]) {
  const int nsites = s.nsites, nfix = s.nfix;
  for (int j = jlo; j <= jhi; ++j) {
    int jtype2 = s.nwtype[std::abs(s.typei[j])];
    for (int i = nsites + 1; i <= j - 1; ++i) {
      int itype2 = s.nwtype[std::abs(s.typei[i])];
      int is = nindex(s, itype2, jtype2);
      double dxx = s.x[i] - s.x[j], dyy = s.y[i] - s.y[j],
             dzz = s.z[i] - s.z[j];
      s.min_image(dxx, dyy, dzz);  // extension mode only
      double dist2 = dxx * dxx + dyy * dyy + dzz * dzz;
      if (s.periodic && dist2 >= s.rcut2) continue;
      double de = 0.0, dist = 0.0, idist = 0.0, idist2 = 0.0, cofo = 0.0,
             dist6 = 0.0, dist12 = 0.0, esrpmf1 = 0.0, esrpmf2 = 0.0,
             esrpmf3 = 0.0, fdf = 0.0, fdv = 0.0, eefp = 0.0;
      if (s.qefpot[is]) {
        if (qforces)
          getyd(s, is, dist2, eefp, de, dist);
        else
          gety(s, is, dist2, eefp, dist);
        e[3] += eefp;
      } else {
        idist2 = 1.0 / dist2;
        if (s.qchr[is] || s.qsrpmfi[is]) idist = std::sqrt(idist2);
        if (s.qchr[is]) {
          cofo = s.fct[is] * idist;
          e[0] += cofo;
        }
        if (s.qlj[is]) {
          dist6 = pow3(s.sgp2[is] * idist2);
          dist12 = dist6 * dist6;
          e[1] += s.epp4[is] * (dist12 - dist6);
        }
        if (s.qsrpmfi[is] && dist2 <= s.rth) {
          dist = 1.0 / idist;
          esrpmf1 = std::exp((s.c1[is] - dist) * s.c2[is]);
          esrpmf2 = std::cos(s.c3[is] * pi * (s.c1[is] - dist));
          esrpmf3 = pow6(s.c1[is] * idist);
          double esrpmf0 = s.c0[is] * esrpmf1 * esrpmf2 + s.c4[is] * esrpmf3;
          if (dist >= s.srpx) {
            fdf = std::exp(-s.srpk * (dist - s.srpx)) - s.srpy;
            fdv = esrpmf0;
            esrpmf0 = fdv * fdf;
          }
          e[2] += esrpmf0;
        }
      }
      if (qforces) {
        if (!s.qefpot[is]) {
          de = 0.0;
          if (s.qchr[is]) de = cofo * idist2;
          if (s.qlj[is])
            de = de + s.epp4[is] * (2.0 * dist12 - dist6) * 6.0 * idist2;
          if (s.qsrpmfi[is] && dist2 <= s.rth) {
            double dc = (-s.c2[is] * esrpmf2 +
                         s.c3[is] * pi *
                             std::sin(s.c3[is] * pi * (s.c1[is] - dist))) *
                            s.c0[is] * esrpmf1 -
                        6.0 * s.c4[is] * esrpmf3 * idist;
            if (dist >= s.srpx) dc = dc * fdf - fdv * s.srpk * (fdf + s.srpy);
            de = de - dc * idist;
          }
        }
        if (de != 0.0) {
          if (i > nsites + nfix) {
            fx[i] += de * dxx;
            fy[i] += de * dyy;
            fz[i] += de * dzz;
          }
          fx[j] -= de * dxx;
          fy[j] -= de * dyy;
          fz[j] -= de * dzz;
        }
      }
    }
  }
}

// ---- ENERGY: energy.mono.f90:19-692 ---------------------------------------
void energy(State &s, uint32_t mask, bool qforces) {
  s.ener = s.eelec = s.eefpot = s.eefpotmx = s.evdw = s.esrpmf = s.esrpmfmx =
      s.ememb = s.egsbpa = s.egsbpb = s.evdwgd = s.eqqmx = s.evdwmx = 0.0;
  s.erfpar = 0.0;
  if (qforces)
    for (int i = 1; i <= s.ntot; ++i) s.fx[i] = s.fy[i] = s.fz[i] = 0.0;

  const bool Qmemb = (mask & BROMOC_M_MEMB) && s.qmemb;
  const bool Qphix = (mask & BROMOC_M_PHIX) && s.qphix;
  const bool Qphiv = (mask & BROMOC_M_PHIV) && s.qphiv;
  const bool Qrfpar = (mask & BROMOC_M_RFPAR) && s.qrfpar;
  const bool Qnonbond = (mask & BROMOC_M_NONBOND) != 0;

  if (Qmemb) membrane(s, qforces);
  s.ener = s.ememb;
  // energy.mono.f90:71-79
  if ((mask & BROMOC_M_MMIJ) && s.mm.on) {
    mmij_energy(s, qforces);
    s.ener += s.egsbpb;
  }
  if (Qphix) {
    staticf1(s, qforces);
    s.ener += s.egsbpa;
  }
  if (Qphiv) {
    if (s.qtrln)
      vdwgd1trln(s, qforces);
    else
      vdwgd1spln(s, qforces);
    s.ener += s.evdwgd;
  }
  if (Qrfpar) {
    rfparion(s, qforces);
    s.ener += s.erfpar;
    s.egsbpb = s.erfpar;
  }

  const int nsites = s.nsites, nfix = s.nfix, ntot = s.ntot;
  // ion-ion: energy.mono.f90:117-194
  if (s.qpar() && Qnonbond) {
    const int jfirst = nsites + nfix + 1;
#ifdef _OPENMP
    // energy.para.f90:120-155: each thread takes a j-range holding an equal
    // share of the triangular pair count and accumulates privately.
    const long aa = (long)(ntot - nsites - nfix) * (ntot - nsites + nfix - 1) / 2;
#pragma omp parallel
    {
      const int nth = omp_get_num_threads(), tid = omp_get_thread_num();
      const double bb = (double)aa / nth;
      int ini = tid == 0 ? jfirst
                         : (int)(std::sqrt(0.25 + 2.0 * bb * tid + nfix * (nfix - 1.0)) +
                                 0.5 + 1 + nsites);
      int fin = tid + 1 == nth
                    ? ntot
                    : (int)(std::sqrt(0.25 + 2.0 * bb * (tid + 1) + nfix * (nfix - 1.0)) +
                            0.5 + nsites);
      std::vector<double> fxl(ntot + 1, 0.0), fyl(ntot + 1, 0.0), fzl(ntot + 1, 0.0);
      double el[4] = {0, 0, 0, 0};
      ionion_range(s, ini, fin, qforces, fxl.data(), fyl.data(), fzl.data(), el);
#pragma omp critical
      {
        s.eelec += el[0];
        s.evdw += el[1];
        s.esrpmf += el[2];
        s.eefpot += el[3];
        if (qforces)
          for (int i = 1; i <= ntot; ++i) {
            s.fx[i] += fxl[i];
            s.fy[i] += fyl[i];
            s.fz[i] += fzl[i];
          }
      }
    }
#else
    double el[4] = {s.eelec, s.evdw, s.esrpmf, s.eefpot};
    ionion_range(s, jfirst, ntot, qforces, s.fx.data(), s.fy.data(),
                 s.fz.data(), el);
    s.eelec = el[0];
    s.evdw = el[1];
    s.esrpmf = el[2];
    s.eefpot = el[3];
#endif
  }
  // DNA bonded and Go-like terms: energy.mono.f90:196-582
  nucl_energy(s, mask, qforces);

  // dids(1:5, nsites+1:ntot) = 0 (energy.mono.f90:583)
  for (int i = nsites + 1; i <= ntot; ++i)
    for (int m = 0; m < 5; ++m) s.dids[5 * (i - 1) + m] = 0.0;
  const bool qproxdiff = s.have_dif && s.dif.diffcutoff > 0.0;
  // ion-site: energy.mono.f90:585-687
  if (s.qpar() && s.qnucl() && Qnonbond) {
    for (int j = 1; j <= nsites; ++j) {
      int jtype2 = s.typtyp[j];
      for (int i = nsites + 1; i <= ntot; ++i) {
        int itype2 = s.nwtype[std::abs(s.typei[i])];
        int is = nindex(s, itype2, jtype2);
        double dxx = s.x[i] - s.x[j], dyy = s.y[i] - s.y[j],
               dzz = s.z[i] - s.z[j];
        double dist2 = dxx * dxx + dyy * dyy + dzz * dzz;
        bool ok2 = qforces && (i > nsites + nfix || s.stfree[j]);
        double de = 0.0, dist = 0.0, idist = 0.0, idist2 = 0.0, cofo = 0.0,
               dist6 = 0.0, dist12 = 0.0, esrpmf1 = 0.0, esrpmf2 = 0.0,
               esrpmf3 = 0.0, fdf = 0.0, fdv = 0.0, eefp = 0.0;
        if (s.qefpot[is]) {
          if (ok2)
            getyd(s, is, dist2, eefp, de, dist);
          else
            gety(s, is, dist2, eefp, dist);
          s.eefpotmx += eefp;
          if (qproxdiff && dist > 0.0) {
            double *d = &s.dids[5 * (i - 1)];
            if (j == 1) {
              d[0] = dist - s.dmi[is];
              d[1] = dist;
              d[2] = dxx;
              d[3] = dyy;
              d[4] = dzz;
            } else {
              double didstmp = dist - s.dmi[is];
              if (didstmp < d[0]) {
                d[0] = didstmp;
                d[1] = dist;
                d[2] = dxx;
                d[3] = dyy;
                d[4] = dzz;
              }
            }
          }
        } else {
          idist2 = 1.0 / dist2;
          if (s.qchr[is] || s.qsrpmfi[is]) idist = std::sqrt(idist2);
          if (s.qchr[is]) {
            cofo = s.fct[is] * idist;
            s.eqqmx += cofo;
          }
          if (s.qlj[is]) {
            dist6 = pow3(s.sgp2[is] * idist2);
            dist12 = dist6 * dist6;
            s.evdwmx += s.epp4[is] * (dist12 - dist6);
          }
          if (s.qsrpmfi[is] && dist2 <= s.rth) {
            dist = 1.0 / idist;
            esrpmf1 = std::exp((s.c1[is] - dist) * s.c2[is]);
            esrpmf2 = std::cos(s.c3[is] * pi * (s.c1[is] - dist));
            esrpmf3 = pow6(s.c1[is] * idist);
            double esrpmf0 = s.c0[is] * esrpmf1 * esrpmf2 + s.c4[is] * esrpmf3;
            if (dist >= s.srpx) {
              fdf = std::exp(-s.srpk * (dist - s.srpx)) - s.srpy;
              fdv = esrpmf0;
              esrpmf0 = fdv * fdf;
            }
            s.esrpmfmx += esrpmf0;
          }
        }
        if (ok2) {
          if (!s.qefpot[is]) {
            de = 0.0;
            if (s.qchr[is]) de = cofo * idist2;
            if (s.qlj[is])
              de = de + s.epp4[is] * (2.0 * dist12 - dist6) * 6.0 * idist2;
            if (s.qsrpmfi[is] && dist2 <= s.rth) {
              double dc = (-s.c2[is] * esrpmf2 +
                           s.c3[is] * pi *
                               std::sin(s.c3[is] * pi * (s.c1[is] - dist))) *
                              s.c0[is] * esrpmf1 -
                          6.0 * s.c4[is] * esrpmf3 * idist;
              if (dist >= s.srpx) dc = dc * fdf - fdv * s.srpk * (fdf + s.srpy);
              de = de - dc * idist;
            }
          }
          if (de != 0.0) {
            if (i > nsites + nfix) {
              s.fx[i] += de * dxx;
              s.fy[i] += de * dyy;
              s.fz[i] += de * dzz;
            }
            if (s.stfree[j]) {
              s.fx[j] -= de * dxx;
              s.fy[j] -= de * dyy;
              s.fz[j] -= de * dzz;
            }
          }
        }
      }
    }
  }
  // energy.mono.f90:689
  s.ener += s.eelec + s.evdw + s.esrpmf + s.esrpmfmx + s.ebond + s.eang + s.edihe +
            s.estack + s.ebp + s.eex + s.eqq + s.esolv + s.eqqmx + s.evdwmx + s.eefpot +
            s.eefpotmx + s.econ;
}

}  // namespace bref
