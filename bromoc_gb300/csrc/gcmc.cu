// INTERACT (interact.f90) and GRAND (grand.f90, insert.f90, find.f90) on the
// device, all in FP64.  A GCMC attempt is three launches with no host round
// trip: proposal + the trial's single-particle terms (1 block) -> pair and
// RFPAR cross sums over the other particles (grid) -> total ΔE + Im-Roux
// acceptance + insertion/deletion (1 block).  The live particle count stays
// on the device (DevState::ntot).
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kIaThreads = 64;
constexpr int kPropThreads = 256;

int interact_slots(int ntot_ub) { return (ntot_ub + kIaThreads - 1) / kIaThreads; }

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double seg8(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// Single-particle terms of INTERACT for the trial, one full warp: lane 0 the
// membrane (interact.f90:59-119), lanes 8g+corner the trilinear nodes of the
// static field (staticf0.f90), repulsion (vdwgd0trln.f90), gsrfen and greff
// (rfpar.f90:312-344 with its early exit); lanes 0..26 the B-spline nodes
// (vdwgd0spln.f90).  Fills e_single, srfe, reff, rf_in of tr (lane 0).
__device__ void trial_single_warp(const KP &p, Trial &tr, uint32_t mask, int qalert) {
  const int lane = threadIdx.x & 31;
  const int j0 = tr.j - 1;
  const bool beion = j0 >= p.nsites;
  const int jt2 = beion ? p.nwtype[tr.itype] : p.typtyp[j0];
  const double charge = beion ? p.cg[tr.itype] : p.sitecharge[j0];
  const double x = tr.x, y = tr.y, z = tr.z;
  const int g = lane >> 3, c = lane & 7;
  const int ca = (c >> 2) & 1, cb = (c >> 1) & 1, cc = c & 1;
  const bool do_phix = (mask & 4u) && p.qphix && (beion || charge != 0.0) &&
                       in_grid(p.g1, x, y, z);
  const Grid3 &g2 = p.g2;
  const bool do_phiv = (mask & 8u) && p.qphiv && x <= g2.xbcen + g2.tranx &&
                       x >= g2.xbcen - g2.tranx && y <= g2.ybcen + g2.trany &&
                       y >= g2.ybcen - g2.trany && z <= p.vzmax && z >= p.vzmin;
  const bool do_rf = (mask & 16u) && p.qrfpar && beion && in_grid(p.g3, x, y, z);
  size_t vifir = 0;
  double esvdw = 0.0;
  int vit2 = 0;
  if (do_phiv) phiv_select(p, j0, beion ? tr.itype : 0, vifir, esvdw, vit2);

  double v = 0.0, psum = 0.0, gs_own = 0.0;
  bool active = false;
  double w = 0.0;
  if ((g == 0 && do_phix) || (g == 1 && do_phiv && p.qtrln) || (g >= 2 && do_rf)) {
    const Grid3 &gg = g == 0 ? p.g1 : (g == 1 ? p.g2 : p.g3);
    const double xi = x + gg.tranx - gg.xbcen, yi = y + gg.trany - gg.ybcen,
                 zi = z + gg.tranz - gg.zbcen;
    int ix, iy, iz;
    cell_of(gg, xi, yi, zi, ix, iy, iz);
    const double ai = 1.0 - fabs(xi - (ix + ca) * gg.dcel) * gg.idcel;
    const double bi = 1.0 - fabs(yi - (iy + cb) * gg.dcel) * gg.idcel;
    const double ci = 1.0 - fabs(zi - (iz + cc) * gg.dcel) * gg.idcel;
    w = ai * bi * ci;
    const size_t node = (size_t)(ix + ca) * gg.ncly * gg.nclz + (size_t)(iy + cb) * gg.nclz +
                        iz + cc;
    if (g == 0) {
      v = (double)__ldg(p.phix + node) * charge * p.celec;
    } else if (g == 1) {
      const double phis = (double)__ldg(p.phiv + vifir + node);
      psum = phis;
      v = esvdw * phis;
    } else {
      const size_t n3 = rfpar_ifir(p, tr.itype) + node;
      gs_own = (double)__ldg(p.gsrfen + n3);
      v = g == 2 ? gs_own : p.sqrfac * (double)__ldg(p.greff + n3);
    }
    active = true;
  }
  const double gs_c0 = __shfl_sync(0xffffffffu, gs_own, lane & ~1);
  if (g >= 2 && active && !(gs_c0 != 0.0 && (cc == 0 || gs_own != 0.0))) active = false;
  double le = active ? w * v : 0.0;
  le = seg8(le);
  psum = seg8(psum);
  double be = 0.0, bsum = 0.0;
  if (do_phiv && !p.qtrln) {  // warp-uniform
    double e1 = 0.0, s1 = 0.0;
    if (lane < 27) {
      const double xi = x + g2.tranx - g2.xbcen, yi = y + g2.trany - g2.ybcen,
                   zi = z + g2.tranz - g2.zbcen;
      int ix, iy, iz;
      spln_cell(g2, xi, yi, zi, ix, iy, iz);
      const int k = ix - 1 + lane / 9, l = iy - 1 + (lane / 3) % 3, m = iz - 1 + lane % 3;
      const double fi = m3(1.5 - (xi - k * g2.dcel) * g2.idcel) *
                        m3(1.5 - (yi - l * g2.dcel) * g2.idcel) *
                        m3(1.5 - (zi - m * g2.dcel) * g2.idcel);
      if (fi != 0.0) {
        const double phis = (double)__ldg(p.phiv + vifir + (size_t)k * g2.ncly * g2.nclz +
                                          (size_t)l * g2.nclz + m);
        s1 = phis;
        e1 = fi * esvdw * phis;
      }
    }
    be = wsum(e1);
    bsum = wsum(s1);
  }
  const double e_v = __shfl_sync(0xffffffffu, le, 8), s_v = __shfl_sync(0xffffffffu, psum, 8);
  const double sj = __shfl_sync(0xffffffffu, le, 16), rj = __shfl_sync(0xffffffffu, le, 24);
  if (lane == 0) {
    double e = 0.0;
    if ((mask & 2u) && p.qmemb) {
      double f[3];
      if (membrane_one(p, jt2, charge, x, y, z, false, true, e, f) && qalert)
        atomicAdd(&p.warn[jt2], 1);
    }
    if (do_rf) e += 0.5 * p.celec * p.cg[tr.itype] * p.cg[tr.itype] * sj * sj;
    if (do_phix) e += le;
    if (do_phiv) {
      double ev = p.qtrln ? e_v : be;
      const double ps = p.qtrln ? s_v : bsum;
      if (ps >= (p.qtrln ? p.thold8 : p.thold27)) {
        ev = 1.0e10;
        if (qalert) atomicAdd(&p.warn[jt2], 1);
      }
      e += ev;
    }
    tr.e_single = e;
    tr.srfe = do_rf ? sj : 0.0;
    tr.reff = do_rf ? rj : 0.0;
    tr.rf_in = do_rf ? 1 : 0;
  }
}

// Partial ΔE over the other particles: pair terms (ion-ion, ion-site) and
// the RFPAR cross term (rfpar.f90:356-367).
__global__ void __launch_bounds__(kIaThreads) k_interact_part(KP p, uint32_t mask) {
  __shared__ double red[kIaThreads / 32];
  __shared__ double tot[1];
  const Trial tr = *p.trial;
  const int ntot = p.st->ntot;
  const int j0 = tr.j - 1;
  // an invalid trial (rejected before INTERACT) carries no slot or type
  const bool beion = tr.valid && j0 >= p.nsites;
  int jt2 = 0;
  if (tr.valid && !guard_bad(p.st, j0, (long long)p.cap + 1, 29))
    jt2 = beion ? p.nwtype[tr.itype] : p.typtyp[j0];
  const bool rf = tr.valid && tr.rf_in;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double u = 0.0;
  int err = 0;
  const bool ion_i = i >= p.nsites;
  bool ok = tr.valid && i < ntot && i != j0 && !guard_bad(p.st, jt2 - 1, p.nttyp, 30);
  if (ok && ion_i)
    ok = !guard_bad(p.st, abs(p.typei[i]) - p.nold - 1, p.ntype - p.nold, 31);
  if (ok) {
    const double dx = p.x[i] - tr.x, dy = p.y[i] - tr.y, dz = p.z[i] - tr.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (mask & 1u) {
      int is = -1;
      if (beion && ion_i)  // interact.f90:173-210
        is = p.pidx[(p.nwtype[abs(p.typei[i])] - 1) * p.nttyp + jt2 - 1];
      else if (beion && !ion_i)  // interact.f90:351-381
        is = p.pidx[(p.typtyp[i] - 1) * p.nttyp + jt2 - 1];
      else if (!beion && ion_i)  // interact.f90:383-413
        is = p.pidx[(p.nwtype[abs(p.typei[i])] - 1) * p.nttyp + jt2 - 1];
      if (is >= 0) u += law_interact64(p, p.pp[is], d2, err);
    }
    if (rf && ion_i && in_grid(p.g3, p.x[i], p.y[i], p.z[i])) {
      double si, ri, d1[3], dd2[3];
      const int it = abs(p.typei[i]);
      rfpar_gather(p, p.x[i], p.y[i], p.z[i], rfpar_ifir(p, it), false, si, ri, d1, dd2);
      if (si != 0.0) {
        const double tau = p.celec * p.cg[tr.itype];
        const double reffij = tr.reff * ri;
        u += tau * p.cg[it] * reffij * tr.srfe * si / sqrt(reffij * reffij + d2);
      }
    }
  }
  if (err) atomicOr(&p.st->err, err);
  block_sum<1>(&u, red, tot);
  if (threadIdx.x == 0) p.ipart[blockIdx.x] = tot[0];
}

// Sum of the partials plus the trial's single-particle part: the full ΔE.
__device__ double interact_total(const KP &p, const Trial &tr, int nblk, double *red,
                                 double *tot) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += p.ipart[b];
  block_sum<1>(&v, red, tot);
  return tr.e_single + tot[0];
}

// INTERACT entry: the host wrote the trial; one warp fills its single part.
__global__ void __launch_bounds__(32) k_interact_prep(KP p, uint32_t mask, int qalert) {
  __shared__ Trial s;
  if (threadIdx.x == 0) s = *p.trial;
  __syncwarp();
  Trial t = s;
  trial_single_warp(p, t, mask, qalert);
  if (threadIdx.x == 0) *p.trial = t;
}

__global__ void __launch_bounds__(kIaThreads)
    k_interact_final(KP p, int nblk, double *out) {
  __shared__ double red[kIaThreads / 32];
  __shared__ double tot[1];
  const Trial tr = *p.trial;
  const double d = interact_total(p, tr, nblk, red, tot);
  if (threadIdx.x == 0) *out = d;
}

void launch_interact(const KP &p, int ntot_ub, uint32_t mask, int qalert,
                     double *dener_dev, cudaStream_t stream) {
  const int nb = interact_slots(ntot_ub + 1);
  k_interact_prep<<<1, 32, 0, stream>>>(p, mask, qalert);
  k_interact_part<<<nb, kIaThreads, 0, stream>>>(p, mask);
  k_interact_final<<<1, kIaThreads, 0, stream>>>(p, nb, dener_dev);
}

// ---------------------------------------------------------------------------
// GCMC proposal (grand.f90:42-86, insert.f90, find.f90) and the trial's
// single-particle terms.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPropThreads)
    k_gcmc_propose(KP p, uint32_t mask, uint64_t seed, uint64_t cycle, uint32_t attempt) {
  __shared__ Trial s;
  __shared__ int counts[kPropThreads];
  if (threadIdx.x == 0) {
    Trial t{};
    uint32_t draw = 0;
    const int nbuf = p.nbuffer;
    const int ntot = p.st->ntot;
    if (gcmc_uniform(seed, cycle, attempt, draw++) < 0.5) {
      const int ib = (int)((double)nbuf * gcmc_uniform(seed, cycle, attempt, draw++)) + 1;
      t.insert = 1;
      t.ib = ib;
      if (ib <= nbuf && p.avnum[ib] > 0.0) {
        t.itype = p.ibfftyp[ib];
        t.j = ntot + 1;
        t.valid = 1;
        bool ok = false;
        for (int it = 0; it < (1 << 20) && !ok; ++it) {
          const double u1 = gcmc_uniform(seed, cycle, attempt, draw++);
          const double u2 = gcmc_uniform(seed, cycle, attempt, draw++);
          const double u3 = gcmc_uniform(seed, cycle, attempt, draw++);
          t.x = p.lx * (u1 - 0.5) + p.cx;
          t.y = p.ly * (u2 - 0.5) + p.cy;
          t.z = p.lzmin[ib] + (p.lzmax[ib] - p.lzmin[ib]) * u3;
          ok = true;
          if (p.shape == 1) {
            const double r2 = (t.x - p.cx) * (t.x - p.cx) + (t.y - p.cy) * (t.y - p.cy) +
                              (t.z - p.cz) * (t.z - p.cz);
            ok = r2 > p.rmin[ib] * p.rmin[ib] && r2 < p.rmax[ib] * p.rmax[ib];
          } else if (p.shape == 2) {
            const double ex = (t.x - p.cx) * p.iecx, ey = (t.y - p.cy) * p.iecy;
            ok = ex * ex + ey * ey < 1.0;
          }
        }
        if (!ok) {  // rejection sampling did not terminate: give up the attempt
          t.valid = 0;
          atomicOr(&p.st->err, kErrFind);
        }
      }
    } else {
      const int ib = (int)((double)nbuf * gcmc_uniform(seed, cycle, attempt, draw++)) + 1;
      const int natb = ib <= nbuf ? p.st->nat[ib - 1] : 0;
      const int ip = (int)((double)natb * gcmc_uniform(seed, cycle, attempt, draw++)) + 1;
      t.insert = 0;
      t.ib = ib;
      if (ib <= nbuf && ip <= natb) {
        t.itype = p.ibfftyp[ib];
        t.valid = 1;
        t.j = ip;  // rank within the buffer; resolved to a slot below
      }
    }
    t.draw = (int)draw;
    s = t;
  }
  __syncthreads();
  // every thread reads the proposal before anyone edits it
  const int valid = s.valid, insert = s.insert, ib = s.ib, rank = s.j;
  __shared__ int found;
  if (threadIdx.x == 0) found = -1;
  __syncthreads();
  if (valid && !insert) {
    // find.f90: the rank-th particle of buffer ib in slot order
    const int ntot = p.st->ntot;
    const int lo = p.nsites + p.nfix;
    const int n = ntot - lo;
    const int per = (n + kPropThreads - 1) / kPropThreads;
    const int a = lo + threadIdx.x * per, b = min(ntot, a + per);
    int c = 0;
    for (int k = a; k < b; ++k) c += (p.ibuffer[k] == ib);
    counts[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {  // exclusive scan, fixed order
      int acc = 0;
      for (int k = 0; k < kPropThreads; ++k) {
        const int v = counts[k];
        counts[k] = acc;
        acc += v;
      }
    }
    __syncthreads();
    const int before = counts[threadIdx.x];
    if (rank > before && rank <= before + c) {  // exactly one thread
      int r = before;
      for (int k = a; k < b; ++k)
        if (p.ibuffer[k] == ib && ++r == rank) {
          found = k;
          break;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int k = found;
      if (k < 0 || guard_bad(p.st, k, ntot, 11)) {
        s.valid = 0;
        atomicOr(&p.st->err, kErrFind);
      } else {
        s.j = k + 1;
        s.x = p.x[k];
        s.y = p.y[k];
        s.z = p.z[k];
      }
    }
    __syncthreads();
  }
  // the trial's single-particle terms (deletion trials raise warnings as
  // INTERACT with Qalert does, insertion trials do not: grand.f90:48,86)
  if (threadIdx.x < 32 && s.valid) {
    Trial t = s;
    trial_single_warp(p, t, mask, t.insert ? 0 : 1);
    if (threadIdx.x == 0) s = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) *p.trial = s;
}

// ---------------------------------------------------------------------------
// ΔE + acceptance + bookkeeping (grand.f90:48-116).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kIaThreads)
    k_gcmc_accept(KP p, int nblk, uint64_t seed, uint64_t cycle, uint32_t attempt) {
  __shared__ double red[kIaThreads / 32];
  __shared__ double tot[1];
  const Trial tr = *p.trial;
  double dener = 0.0;
  if (tr.valid) dener = interact_total(p, tr, nblk, red, tot);
  if (threadIdx.x != 0) return;
  DevState *st = p.st;
  if (tr.valid && !guard_bad(st, tr.ib - 1, p.nbuffer, 21)) {
    const int ib = tr.ib, b = ib - 1;
    const int nat = st->nat[b];
    const double boltz = exp(-(dener - p.mu[ib]) * p.ikbt);
    double rate;
    if (tr.insert) {
      if (p.qbufferbias[ib]) {
        rate = p.avnum[ib] + p.kbb[ib] * (p.avnum[ib] - (double)(st->ntotat[b] / (long long)cycle));
        rate = rate * boltz / (double)(nat + 1);
      } else {
        rate = (p.avnum[ib] / (nat + 1)) * boltz;
      }
      rate = rate / (1.0 + rate);
    } else {
      if (p.qbufferbias[ib]) {
        rate = p.avnum[ib] + p.kbb[ib] * (p.avnum[ib] - (double)(st->ntotat[b] / (long long)cycle));
        rate = rate * boltz / (double)nat;
      } else {
        rate = (p.avnum[ib] / nat) * boltz;
      }
      rate = 1.0 / (1.0 + rate);
    }
    if (gcmc_uniform(seed, cycle, attempt, (uint32_t)tr.draw) <= rate) {
      const int ntot = st->ntot;
      if (tr.insert) {
        if (ntot + 1 > p.cap) {
          st->err |= kErrCapacity;
        } else if (!guard_bad(st, ntot, p.cap, 22)) {
          st->dener_sum += dener;
          st->nat[b] = nat + 1;
          p.x[ntot] = tr.x;
          p.y[ntot] = tr.y;
          p.z[ntot] = tr.z;
          p.typei[ntot] = tr.z < p.cz ? -tr.itype : tr.itype;
          p.ibuffer[ntot] = ib;
          st->ntot = ntot + 1;
          st->ninsert[b] += 1;
        }
      } else if (!guard_bad(st, tr.j - 1, ntot, 23) &&
                 !guard_bad(st, ntot - 1, p.cap, 24)) {
        const int iat = tr.j - 1, last = ntot - 1;
        st->dener_sum -= dener;
        st->nremove[b] += 1;
        p.x[iat] = p.x[last];
        p.y[iat] = p.y[last];
        p.z[iat] = p.z[last];
        p.typei[iat] = p.typei[last];
        p.ibuffer[iat] = p.ibuffer[last];
        st->nat[b] = nat - 1;
        st->ntot = ntot - 1;
      }
    }
  }
  for (int b = 0; b < p.nbuffer; ++b)  // prob(ib, nat(ib)) += 1
    if (!guard_bad(st, st->nat[b], p.cap + 1, 25))
      p.prob[(size_t)b * (p.cap + 1) + st->nat[b]] += 1;
}

void launch_gcmc_attempt(const KP &p, int ntot_ub, uint32_t mask, uint64_t seed,
                         uint64_t cycle, uint32_t attempt, cudaStream_t stream) {
  k_gcmc_propose<<<1, kPropThreads, 0, stream>>>(p, mask, seed, cycle, attempt);
  const int nb = interact_slots(ntot_ub + 1);
  k_interact_part<<<nb, kIaThreads, 0, stream>>>(p, mask);
  k_gcmc_accept<<<1, kIaThreads, 0, stream>>>(p, nb, seed, cycle, attempt);
}

}  // namespace bgpu
