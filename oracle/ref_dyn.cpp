// ORACLE -- test infrastructure only (see ref_state.h).
// BD position update, wall handling, crossing counters and GCMC.
#include <cmath>

#include "ref_state.h"

namespace bref {

static inline double fsign(double a, double b) {
  return b >= 0.0 ? std::fabs(a) : -std::fabs(a);
}

// One periodic wrap into [lo, lo + L): BD moves are far shorter than a box.
static inline void wrap1(double lo, double L, double &v) {
  if (v < lo)
    v += L;
  else if (v >= lo + L)
    v -= L;
}

// fixcoor.f90:19-68; in the extension mode (periodic box) the position is
// wrapped into the box instead of clamped.
void fixcoor(const State &s, double &xi, double &yi, double &zi) {
  if (s.periodic) {
    wrap1(s.lx2m, s.sys.lx, xi);
    wrap1(s.ly2m, s.sys.ly, yi);
    wrap1(s.lz2m, s.sys.lz, zi);
    return;
  }
  const bromoc_system &q = s.sys;
  if (q.shape == BROMOC_SPHERE) {
    double r2 = (xi - q.cx) * (xi - q.cx) + (yi - q.cy) * (yi - q.cy) +
                (zi - q.cz) * (zi - q.cz);
    if (r2 > s.rsphe2) {
      double lzrad = 2.0 * q.rsphe / std::sqrt(r2) - 1.0;
      xi = lzrad * (xi - q.cx) + q.cx;
      yi = lzrad * (yi - q.cy) + q.cy;
      zi = lzrad * (zi - q.cz) + q.cz;
    }
  } else if (q.shape == BROMOC_ECYL) {
    double ex = (xi - q.cx) * s.iecx, ey = (yi - q.cy) * s.iecy;
    double r2 = ex * ex + ey * ey;
    if (r2 > 1.0) {
      double r = 0.999999999999999 / std::sqrt(r2);
      xi = r * (xi - q.cx) + q.cx;
      yi = r * (yi - q.cy) + q.cy;
    }
    if (zi < s.lz2m)
      zi = s.lz2m;
    else if (zi > s.lz2p)
      zi = s.lz2p;
  } else {
    if (xi < s.lx2m)
      xi = s.lx2m;
    else if (xi > s.lx2p)
      xi = s.lx2p;
    if (yi < s.ly2m)
      yi = s.ly2m;
    else if (yi > s.ly2p)
      yi = s.ly2p;
    if (zi < s.lz2m)
      zi = s.lz2m;
    else if (zi > s.lz2p)
      zi = s.lz2p;
  }
}

// countions.f90:19-32
static void countions(State &s, double zold, double zi, int it) {
  for (int j = 1; j <= s.cntpts; ++j) {
    int k = (it - 1) * s.cntpts + (j - 1);
    if (zold < s.zcont[j] && zi >= s.zcont[j])
      s.nforward[k] += 1;
    else if (zold >= s.zcont[j] && zi < s.zcont[j])
      s.nbackward[k] += 1;
  }
}

// sevalmod.f90:23-65 (interval by bisection; the cached interval of the
// reference returns the same piece except exactly at a knot, where the
// spline is continuous)
static int seval_interval(int n, double u, const std::vector<double> &x) {
  int i = 1, j = n + 1;
  do {
    int k = (i + j) / 2;
    if (u < x[k]) j = k;
    if (u >= x[k]) i = k;
  } while (j > i + 1);
  return i;
}

static void clamp_bd(double bdmax, double &d) {
  if (std::fabs(d) > bdmax) d = fsign(bdmax, d);
}

// dynamics0/1/2/3.mono.f90 (+ dynamics0nuc.f90 for DNA sites)
void dynamics(State &s, int variant, uint64_t seed, uint64_t step) {
  const bromoc_system &q = s.sys;
  const double bdmax = q.bdmax, dt = q.dt;
  // dynamics0nuc(1, nsites): free sites move first in the slot order
  for (int i = 1; i <= s.nsites; ++i) {
    if (!s.stfree[i]) continue;
    double delx = s.fx[i] * s.dif.fact0n1, dely = s.fy[i] * s.dif.fact0n1,
           delz = s.fz[i] * s.dif.fact0n1;
    clamp_bd(bdmax, delx);
    clamp_bd(bdmax, dely);
    clamp_bd(bdmax, delz);
    uint32_t slot = (uint32_t)(i - 1);
    s.x[i] += delx + s.dif.fact0n2 * bd_gauss(seed, step, slot, 0);
    s.y[i] += dely + s.dif.fact0n2 * bd_gauss(seed, step, slot, 1);
    s.z[i] += delz + s.dif.fact0n2 * bd_gauss(seed, step, slot, 2);
    if (!s.dif.qdnafree) fixcoor(s, s.x[i], s.y[i], s.z[i]);
  }
  for (int i = s.nsites + s.nfix + 1; i <= s.ntot; ++i) {
    int itype = std::abs(s.typei[i]);
    double fact1, fact2, dDx = 0.0, dDy = 0.0, dDz = 0.0;
    if (variant == BROMOC_DYN1) {
      // dynamics1.mono.f90:39-72
      double zz = s.z[i], pp3 = s.p3[itype];
      double pore1 = -s.dif.plength2 + s.dif.pcenter;
      double pore2 = s.dif.plength2 + s.dif.pcenter;
      double sw, dsw;
      if (zz > pore1 - pp3 && zz < pore2 + pp3) {
        if (zz >= pore1 && zz <= pore2) {
          sw = 0.0;
          dsw = 0.0;
        } else {
          double ipp3 = 1.0 / pp3;
          sw = 0.0;
          dsw = 0.0;
          if (zz > pore2) {
            double d = (zz - pore2) * ipp3;
            sw = 2.0 * d * d * d - 3.0 * d * d;
            dsw = 6.0 * (d * d - d) * ipp3;
          } else if (zz < pore1) {
            double d = (zz - pore1) * ipp3;
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
      double idif = s.diffusion[itype] * (s.ampl3[itype] + (1.0 - s.ampl3[itype]) * sw);
      double didif = s.diffusion[itype] * (1.0 - s.ampl3[itype]) * dsw;
      fact1 = idif * s.kbtdt;
      fact2 = std::sqrt(2.0 * dt * idif);
      dDz = didif * dt;
    } else if (variant == BROMOC_DYN2) {
      // dynamics2.mono.f90:41-74
      const int n = s.dif.nspline;
      double zz = s.z[i], sw = 0.0, dsw = 0.0;
      bool inside = false;
      if (s.xs[1] < s.xs[n]) {
        if (zz < s.xs[1]) {
          sw = s.ys[1];
        } else if (zz > s.xs[n]) {
          sw = s.ys[n];
        } else {
          inside = true;
        }
      } else if (s.xs[1] > s.xs[n]) {
        if (zz > s.xs[1]) {
          sw = s.ys[1];
        } else if (zz < s.xs[n]) {
          sw = s.ys[n];
        } else {
          inside = true;
        }
      }
      if (inside) {
        int k = seval_interval(n, zz, s.xs);
        double dx = zz - s.xs[k];
        sw = s.ys[k] + dx * (s.sb[k] + dx * (s.scc[k] + dx * s.sd[k]));
        dsw = s.sb[k] + dx * (s.scc[k] + dx * s.sd[k]);
      }
      double idif = s.diffusion[itype] * sw;
      double didif = s.diffusion[itype] * dsw;
      fact1 = idif * s.kbtdt;
      fact2 = std::sqrt(2.0 * dt * idif);
      dDz = didif * dt;
    } else if (variant == BROMOC_DYN3) {
      // dynamics3.mono.f90:40-59
      const double *d = &s.dids[5 * (i - 1)];
      if (d[0] > 0.0 && d[0] <= s.dif.diffcutoff) {
        double ebet = std::exp(-d[0] * s.dif.ibeta);
        double idif = s.diffusion[itype] - (s.diffusion[itype] - s.dif.diff0) * ebet;
        double didif = (s.diffusion[itype] - s.dif.diff0) * s.dif.ibeta * ebet;
        double idist = 1.0 / d[1];
        fact1 = idif * s.kbtdt;
        fact2 = std::sqrt(2.0 * dt * idif);
        dDx = didif * dt * d[2] * idist;
        dDy = didif * dt * d[3] * idist;
        dDz = didif * dt * d[4] * idist;
      } else {
        fact1 = s.fact1a[itype];
        fact2 = s.fact2a[itype];
      }
    } else {
      fact1 = s.fact1a[itype];
      fact2 = s.fact2a[itype];
    }
    double delx = s.fx[i] * fact1, dely = s.fy[i] * fact1, delz = s.fz[i] * fact1;
    clamp_bd(bdmax, delx);
    clamp_bd(bdmax, dely);
    clamp_bd(bdmax, delz);
    uint32_t slot = (uint32_t)(i - 1);
    double zold = s.z[i];
    s.x[i] += delx + fact2 * bd_gauss(seed, step, slot, 0) + dDx;
    s.y[i] += dely + fact2 * bd_gauss(seed, step, slot, 1) + dDy;
    s.z[i] += delz + fact2 * bd_gauss(seed, step, slot, 2) + dDz;
    if (q.qcountion) countions(s, zold, s.z[i], itype - s.nold);
    fixcoor(s, s.x[i], s.y[i], s.z[i]);
  }
  // NOTRAN (simul1.f90:380-385): x(1:nsites) = x(1:nsites) -
  // sum(x(1:nsites))*insites + notrx along each flagged axis
  const Nucl &n = s.nuc;
  if (n.on && s.nsites > 0) {
    const double insites = 1.0 / s.nsites;
    std::vector<double> *pos[3] = {&s.x, &s.y, &s.z};
    for (int a = 0; a < 3; ++a) {
      if (!n.qnotr[a]) continue;
      std::vector<double> &v = *pos[a];
      double sm = 0.0;
      for (int i = 1; i <= s.nsites; ++i) sm = sm + v[i];
      for (int i = 1; i <= s.nsites; ++i) v[i] = v[i] - sm * insites + n.notr[a];
    }
  }
}

// insert.f90:19-44.  Uniform draws come from the attempt's stream.
static void insert(State &s, int ib, double &xnew, double &ynew, double &znew,
                   uint64_t seed, uint64_t icycle, uint32_t attempt,
                   uint32_t &draw) {
  const bromoc_system &q = s.sys;
  bool ok = false;
  while (!ok) {
    xnew = q.lx * (gcmc_uniform(seed, icycle, attempt, draw++) - 0.5) + q.cx;
    ynew = q.ly * (gcmc_uniform(seed, icycle, attempt, draw++) - 0.5) + q.cy;
    znew = s.lzmin[ib] +
           (s.lzmax[ib] - s.lzmin[ib]) * gcmc_uniform(seed, icycle, attempt, draw++);
    ok = true;
    if (q.shape == BROMOC_SPHERE) {
      double r2 = (xnew - q.cx) * (xnew - q.cx) + (ynew - q.cy) * (ynew - q.cy) +
                  (znew - q.cz) * (znew - q.cz);
      ok = r2 > s.rmin[ib] * s.rmin[ib] && r2 < s.rmax[ib] * s.rmax[ib];
    } else if (q.shape == BROMOC_ECYL) {
      double ex = (xnew - q.cx) * s.iecx, ey = (ynew - q.cy) * s.iecy;
      ok = ex * ex + ey * ey < 1.0;
    }
  }
}

// find.f90:19-35
static int find(const State &s, int ib, int nini, int ip) {
  int ipx = 0, iat;
  for (iat = nini + 1; iat <= s.ntot; ++iat) {
    if (s.ibuffer[iat] == ib) {
      ipx += 1;
      if (ip == ipx) return iat;
    }
  }
  return iat;  // the Fortran do-variable after loop exhaustion
}

// count.f90:19-95: each mobile ion's buffer (the first whose ion type and
// z range -- and for a sphere the radial shell -- hold it), nat, the sign of
// a buffer ion's type by its side of cz, then ntotat += nat.  A particle
// outside the system is the reference's fatal error: false.
bool count(State &s) {
  const bromoc_system &q = s.sys;
  for (int ib = 1; ib <= s.nbuffer; ++ib) s.nat[ib] = 0;
  bool ok = true;
  for (int i = s.nsites + 1; i <= s.ntot; ++i) {
    s.ibuffer[i] = 0;
    if (i <= s.nsites + s.nfix) continue;
    const int itype = std::abs(s.typei[i]);
    bool endlog = false;
    for (int ib = 1; ib <= s.nbuffer && !endlog; ++ib) {
      if (itype != s.ibfftyp[ib] || !(s.z[i] >= s.lzmin[ib] && s.z[i] <= s.lzmax[ib])) continue;
      if (q.shape == BROMOC_SPHERE) {
        const double r2 = (s.x[i] - q.cx) * (s.x[i] - q.cx) + (s.y[i] - q.cy) * (s.y[i] - q.cy) +
                          (s.z[i] - q.cz) * (s.z[i] - q.cz);
        if (r2 > s.rsphe2) ok = false;
        if (!(r2 >= s.rmin[ib] * s.rmin[ib] && r2 <= s.rmax[ib] * s.rmax[ib])) continue;
      } else {
        if (q.shape == BROMOC_ECYL) {
          const double ex = (s.x[i] - q.cx) * s.iecx, ey = (s.y[i] - q.cy) * s.iecy;
          if (ex * ex + ey * ey > 1.0) ok = false;
        } else if (s.x[i] < s.lx2m || s.x[i] > s.lx2p || s.y[i] < s.ly2m || s.y[i] > s.ly2p) {
          ok = false;
        }
        if (s.z[i] < s.lz2m || s.z[i] > s.lz2p) ok = false;
      }
      s.ibuffer[i] = ib;
      s.nat[ib] += 1;
      s.typei[i] = s.z[i] < q.cz ? -itype : itype;
      endlog = true;
    }
  }
  for (int ib = 1; ib <= s.nbuffer; ++ib) s.ntotat[ib] += s.nat[ib];
  return ok;
}

// grand.f90:19-121
void grand(State &s, uint32_t mask, int ngcmc, uint64_t seed, uint64_t icycle,
           double &dener_sum) {
  const double nbufferr = (double)s.nbuffer;
  dener_sum = 0.0;
  for (int igrand = 1; igrand <= ngcmc; ++igrand) {
    uint32_t attempt = (uint32_t)(igrand - 1), draw = 0;
    if (gcmc_uniform(seed, icycle, attempt, draw++) < 0.5) {
      int ib = (int)(nbufferr * gcmc_uniform(seed, icycle, attempt, draw++)) + 1;
      if (ib <= s.nbuffer && s.avnum[ib] > 0.0) {
        int itype = s.ibfftyp[ib];
        double xnew, ynew, znew, dener;
        insert(s, ib, xnew, ynew, znew, seed, icycle, attempt, draw);
        interact(s, mask, dener, xnew, ynew, znew, itype, s.ntot + 1, false);
        double rate;
        if (s.qbufferbias[ib]) {
          rate = s.avnum[ib] + s.kb[ib] * (s.avnum[ib] - (double)(s.ntotat[ib] / (int64_t)icycle));
          rate = rate * std::exp(-(dener - s.mu[ib]) * s.ikbt) / (double)(s.nat[ib] + 1);
        } else {
          rate = (s.avnum[ib] / (s.nat[ib] + 1)) * std::exp(-(dener - s.mu[ib]) * s.ikbt);
        }
        rate = rate / (1.0 + rate);
        if (gcmc_uniform(seed, icycle, attempt, draw++) <= rate) {
          if (s.ntot + 1 > s.capacity) {
            s.err = "grand: ntot is greater than datom";
            return;
          }
          dener_sum += dener;
          s.nat[ib] += 1;
          s.ntot += 1;
          s.x[s.ntot] = xnew;
          s.y[s.ntot] = ynew;
          s.z[s.ntot] = znew;
          s.typei[s.ntot] = itype;
          if (znew < s.sys.cz) s.typei[s.ntot] = -itype;
          s.ibuffer[s.ntot] = ib;
          s.ninsert[ib] += 1;
        }
      }
    } else {
      int ib = (int)(nbufferr * gcmc_uniform(seed, icycle, attempt, draw++)) + 1;
      // nat(ib) for ib == nbuffer+1 is read out of range in the reference;
      // ip is then unused because ib > nbuffer rejects the attempt.
      int natb = ib <= s.nbuffer ? s.nat[ib] : 0;
      int ip = (int)((double)natb * gcmc_uniform(seed, icycle, attempt, draw++)) + 1;
      if (ib <= s.nbuffer && ip <= s.nat[ib]) {
        int itype = s.ibfftyp[ib];
        int iat = find(s, ib, s.nfix + s.nsites, ip);
        double dener;
        interact(s, mask, dener, s.x[iat], s.y[iat], s.z[iat], itype, iat, true);
        double rate;
        if (s.qbufferbias[ib]) {
          rate = s.avnum[ib] + s.kb[ib] * (s.avnum[ib] - (double)(s.ntotat[ib] / (int64_t)icycle));
          rate = rate * std::exp(-(dener - s.mu[ib]) * s.ikbt) / (double)s.nat[ib];
        } else {
          rate = (s.avnum[ib] / s.nat[ib]) * std::exp(-(dener - s.mu[ib]) * s.ikbt);
        }
        rate = 1.0 / (1.0 + rate);
        if (gcmc_uniform(seed, icycle, attempt, draw++) <= rate) {
          dener_sum -= dener;
          s.nremove[ib] += 1;
          s.x[iat] = s.x[s.ntot];
          s.y[iat] = s.y[s.ntot];
          s.z[iat] = s.z[s.ntot];
          s.typei[iat] = s.typei[s.ntot];
          s.ibuffer[iat] = s.ibuffer[s.ntot];
          s.nat[ib] -= 1;
          s.ntot -= 1;
        }
      }
    }
    for (int ib = 1; ib <= s.nbuffer; ++ib)
      s.prob[(size_t)(ib - 1) * (s.capacity + 1) + s.nat[ib]] += 1;
  }
}

// move.f90:19-45: a mobile ion and a displacement of up to mcmax/2 per
// axis, drawn again while the new position lies outside the system.
static bool mc_move(const State &s, double mcmax, uint64_t seed, uint64_t cycle, uint32_t m,
                    uint32_t &draw, int &iat, double &xn, double &yn, double &zn) {
  const bromoc_system &q = s.sys;
  const double natom2 = (double)(s.ntot - s.nsites);
  for (int t = 0; t < kMcTries; ++t) {
    iat = s.nsites + s.nfix + (int)(natom2 * mc_uniform(seed, cycle, m, draw++)) + 1;
    xn = s.x[iat] + mcmax * (mc_uniform(seed, cycle, m, draw++) - 0.5);
    yn = s.y[iat] + mcmax * (mc_uniform(seed, cycle, m, draw++) - 0.5);
    zn = s.z[iat] + mcmax * (mc_uniform(seed, cycle, m, draw++) - 0.5);
    bool out;
    if (q.shape == BROMOC_SPHERE) {
      const double r2 = (xn - q.cx) * (xn - q.cx) + (yn - q.cy) * (yn - q.cy) +
                        (zn - q.cz) * (zn - q.cz);
      out = r2 > s.rsphe2;
    } else if (q.shape == BROMOC_ECYL) {
      const double ex = (xn - q.cx) * s.iecx, ey = (yn - q.cy) * s.iecy;
      out = ex * ex + ey * ey > 1.0 || zn < s.lz2m || zn > s.lz2p;
    } else {
      out = xn < s.lx2m || xn > s.lx2p || yn < s.ly2m || yn > s.ly2p || zn < s.lz2m ||
            zn > s.lz2p;
    }
    if (!out) return true;
  }
  return false;
}

// metropolis.f90:31-55: INTERACT of the ion at its old (with alerts) and new
// position; downhill moves are taken, uphill ones with probability
// exp(-(enew - eold)/kT).
void metropolis(State &s, uint32_t mask, int nmcm, double mcmax, uint64_t seed,
                uint64_t cycle, double &dener_sum, int &naccept) {
  for (int m = 0; m < nmcm; ++m) {
    uint32_t draw = 0;
    int iat = 0;
    double xn, yn, zn;
    if (!mc_move(s, mcmax, seed, cycle, (uint32_t)m, draw, iat, xn, yn, zn)) continue;
    const int it = std::abs(s.typei[iat]);
    double eold, enew;
    interact(s, mask, eold, s.x[iat], s.y[iat], s.z[iat], it, iat, true);
    interact(s, mask, enew, xn, yn, zn, it, iat, false);
    bool acc = enew <= eold;
    if (!acc) acc = mc_uniform(seed, cycle, (uint32_t)m, draw++) < std::exp(-(enew - eold) * s.ikbt);
    if (acc) {
      s.x[iat] = xn;
      s.y[iat] = yn;
      s.z[iat] = zn;
      dener_sum += enew - eold;
      ++naccept;
    }
  }
}

}  // namespace bref
