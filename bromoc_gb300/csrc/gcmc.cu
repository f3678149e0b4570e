// INTERACT (interact.f90) and GRAND (grand.f90, insert.f90, find.f90) on the
// device, all in FP64.  A GCMC attempt is three launches with no host round
// trip: proposal (1 block) -> partial ΔE (grid over particles) -> final ΔE +
// Im-Roux acceptance + insertion/deletion (1 block).  The live particle count
// stays on the device (DevState::ntot).
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kIaThreads = 128;
constexpr int kPropThreads = 256;

int interact_slots(int ntot_ub) { return (ntot_ub + kIaThreads - 1) / kIaThreads; }

// RFPAR gather of the trial particle (no derivatives).
__device__ __forceinline__ void trial_rfpar(const KP &p, const Trial &tr,
                                            double &sj, double &rj, bool &in) {
  sj = rj = 0.0;
  in = in_grid(p.g3, tr.x, tr.y, tr.z);
  if (in) {
    double d1[3], d2[3];
    rfpar_gather(p, tr.x, tr.y, tr.z, rfpar_ifir(p, tr.itype), false, sj, rj,
                 d1, d2);
  }
}

// Partial ΔE over the other particles: pair terms (ion-ion, ion-site) and
// the RFPAR cross term (rfpar.f90:356-367).
__global__ void __launch_bounds__(kIaThreads) k_interact_part(KP p, uint32_t mask) {
  __shared__ double red[kIaThreads / 32];
  __shared__ double s_sj, s_rj;
  __shared__ int s_in;
  const Trial tr = *p.trial;
  const int ntot = p.st->ntot;
  const int j0 = tr.j - 1;
  // an invalid trial (rejected before INTERACT) carries no slot or type
  const bool beion = tr.valid && j0 >= p.nsites;
  int jt2 = 0;
  if (tr.valid && !guard_bad(p.st, j0, (long long)p.cap + 1, 29))
    jt2 = beion ? p.nwtype[tr.itype] : p.typtyp[j0];
  const bool rf = (mask & 16u) && p.qrfpar && beion;
  if (threadIdx.x == 0) {
    double sj = 0, rj = 0;
    bool in = false;
    if (tr.valid && rf) trial_rfpar(p, tr, sj, rj, in);
    s_sj = sj;
    s_rj = rj;
    s_in = in;
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double u = 0.0;
  int err = 0;
  const bool ion_i = i >= p.nsites;
  bool ok = tr.valid && i < ntot && i != j0 &&
            !guard_bad(p.st, jt2 - 1, p.nttyp, 30);
  if (ok && ion_i)
    ok = !guard_bad(p.st, abs(p.typei[i]) - p.nold - 1, p.ntype - p.nold, 31);
  if (ok) {
    const double dx = p.x[i] - tr.x, dy = p.y[i] - tr.y, dz = p.z[i] - tr.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (mask & 1u) {
      if (beion && ion_i) {  // interact.f90:173-210
        const int is = p.pidx[(p.nwtype[abs(p.typei[i])] - 1) * p.nttyp + jt2 - 1];
        u += law_interact64(p, p.pp[is], d2, err);
      } else if (beion && !ion_i) {  // interact.f90:351-381
        const int is = p.pidx[(p.typtyp[i] - 1) * p.nttyp + jt2 - 1];
        u += law_interact64(p, p.pp[is], d2, err);
      } else if (!beion && ion_i) {  // interact.f90:383-413
        const int is = p.pidx[(p.nwtype[abs(p.typei[i])] - 1) * p.nttyp + jt2 - 1];
        u += law_interact64(p, p.pp[is], d2, err);
      }
    }
    if (rf && s_in && ion_i && in_grid(p.g3, p.x[i], p.y[i], p.z[i])) {
      double si, ri, d1[3], dd2[3];
      const int it = abs(p.typei[i]);
      rfpar_gather(p, p.x[i], p.y[i], p.z[i], rfpar_ifir(p, it), false, si, ri,
                   d1, dd2);
      if (si != 0.0) {
        const double tau = p.celec * p.cg[tr.itype];
        const double reffij = s_rj * ri;
        u += tau * p.cg[it] * reffij * s_sj * si / sqrt(reffij * reffij + d2);
      }
    }
  }
  if (err) atomicOr(&p.st->err, err);
  __shared__ double tot[1];
  block_sum<1>(&u, red, tot);
  if (threadIdx.x == 0) p.ipart[blockIdx.x] = tot[0];
}

// Single-particle terms of the trial + sum of the partials: the full ΔE.
__device__ double interact_final(const KP &p, const Trial &tr, uint32_t mask,
                                 int nblk, int qalert, double *red) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += p.ipart[b];
  __shared__ double tot[1];
  block_sum<1>(&v, red, tot);
  if (threadIdx.x != 0) return 0.0;
  const double pairs = tot[0];
  const int j0 = tr.j - 1;
  const bool beion = j0 >= p.nsites;
  const int jt2 = beion ? p.nwtype[tr.itype] : p.typtyp[j0];
  const double charge = beion ? p.cg[tr.itype] : p.sitecharge[j0];
  double dener = 0.0;
  if ((mask & 2u) && p.qmemb) {  // interact.f90:59-119
    double e = 0.0, f[3];
    if (membrane_one(p, jt2, charge, tr.x, tr.y, tr.z, false, true, e, f) && qalert)
      atomicAdd(&p.warn[jt2], 1);
    dener = e;
  }
  if ((mask & 16u) && p.qrfpar && beion) {  // rfpar.f90:350-354 self part
    double sj, rj;
    bool in;
    trial_rfpar(p, tr, sj, rj, in);
    if (in) dener += 0.5 * p.celec * p.cg[tr.itype] * p.cg[tr.itype] * sj * sj;
  }
  if ((mask & 4u) && p.qphix && (beion || charge != 0.0)) {  // staticf0.f90
    double e = 0.0, f[3];
    staticf_one(p, tr.x, tr.y, tr.z, charge, false, e, f);
    dener += e;
  }
  if ((mask & 8u) && p.qphiv) {  // vdwgd0trln.f90 / vdwgd0spln.f90
    const Grid3 &g = p.g2;
    const bool ok = tr.x <= g.xbcen + g.tranx && tr.x >= g.xbcen - g.tranx &&
                    tr.y <= g.ybcen + g.trany && tr.y >= g.ybcen - g.trany &&
                    tr.z <= p.vzmax && tr.z >= p.vzmin;
    if (ok) {
      size_t ifir;
      double esvdw;
      int it2;
      phiv_select(p, j0, beion ? tr.itype : 0, ifir, esvdw, it2);
      const double xi = tr.x + g.tranx - g.xbcen, yi = tr.y + g.trany - g.ybcen,
                   zi = tr.z + g.tranz - g.zbcen;
      double e = 0.0, f[3] = {0, 0, 0};
      if (p.qtrln) {
        if (vdwgd_trln_one(p, xi, yi, zi, ifir, esvdw, false, e, f) >= p.thold8) {
          e = 1.0e10;
          if (qalert) atomicAdd(&p.warn[jt2], 1);
        }
      } else {
        if (vdwgd_spln0(p, xi, yi, zi, ifir, esvdw, e) >= p.thold27) {
          e = 1.0e10;
          if (qalert) atomicAdd(&p.warn[jt2], 1);
        }
      }
      dener += e;
    }
  }
  return dener + pairs;
}

__global__ void __launch_bounds__(kIaThreads)
    k_interact_final(KP p, uint32_t mask, int nblk, int qalert, double *out) {
  __shared__ double red[kIaThreads / 32];
  const Trial tr = *p.trial;
  const double d = interact_final(p, tr, mask, nblk, qalert, red);
  if (threadIdx.x == 0) *out = d;
}

void launch_interact(const KP &p, int ntot_ub, uint32_t mask, int qalert,
                     double *dener_dev, cudaStream_t stream) {
  const int nb = interact_slots(ntot_ub + 1);
  k_interact_part<<<nb, kIaThreads, 0, stream>>>(p, mask);
  k_interact_final<<<1, kIaThreads, 0, stream>>>(p, mask, nb, qalert, dener_dev);
}

// ---------------------------------------------------------------------------
// GCMC proposal (grand.f90:42-86, insert.f90, find.f90).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPropThreads)
    k_gcmc_propose(KP p, uint64_t seed, uint64_t cycle, uint32_t attempt) {
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
            const double r2 = (t.x - p.cx) * (t.x - p.cx) +
                              (t.y - p.cy) * (t.y - p.cy) +
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
  if (threadIdx.x == 0) *p.trial = s;
}

// ---------------------------------------------------------------------------
// ΔE + acceptance + bookkeeping (grand.f90:48-116).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kIaThreads)
    k_gcmc_accept(KP p, uint32_t mask, int nblk, uint64_t seed, uint64_t cycle,
                  uint32_t attempt) {
  __shared__ double red[kIaThreads / 32];
  const Trial tr = *p.trial;
  double dener = 0.0;
  if (tr.valid) dener = interact_final(p, tr, mask, nblk, tr.insert ? 0 : 1, red);
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

void launch_gcmc_attempt(const KP &p, int ntot_ub, uint32_t mask,
                         uint64_t seed, uint64_t cycle, uint32_t attempt,
                         cudaStream_t stream) {
  k_gcmc_propose<<<1, kPropThreads, 0, stream>>>(p, seed, cycle, attempt);
  const int nb = interact_slots(ntot_ub + 1);
  k_interact_part<<<nb, kIaThreads, 0, stream>>>(p, mask);
  k_gcmc_accept<<<1, kIaThreads, 0, stream>>>(p, mask, nb, seed, cycle, attempt);
}

}  // namespace bgpu
