// INTERACT (interact.f90) and GRAND (grand.f90, insert.f90, find.f90) on the
// device, all in FP64.  INTERACT alone is four launches (RFPAR prepass, the
// trial's single-particle terms, the O(N) sum, the total); GRAND runs all
// its attempts in one cooperative launch (k_grand).  The live particle count
// stays on the device (DevState::ntot).
#include <algorithm>

#include "gridsync.cuh"
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kIaThreads = 64;

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
// nalert: when given, the warnings are counted there (lane 0) instead of
// being added to p.warn.
__device__ void trial_single_warp(const KP &p, Trial &tr, uint32_t mask, int qalert,
                                  int *nalert = nullptr) {
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
      if (membrane_one(p, jt2, charge, x, y, z, false, true, e, f) && qalert) {
        if (nalert)
          ++*nalert;
        else
          atomicAdd(&p.warn[jt2], 1);
      }
    }
    if (do_rf) e += 0.5 * p.celec * p.cg[tr.itype] * p.cg[tr.itype] * sj * sj;
    if (do_phix) e += le;
    if (do_phiv) {
      double ev = p.qtrln ? e_v : be;
      const double ps = p.qtrln ? s_v : bsum;
      if (ps >= (p.qtrln ? p.thold8 : p.thold27)) {
        ev = 1.0e10;
        if (qalert) {
          if (nalert)
            ++*nalert;
          else
            atomicAdd(&p.warn[jt2], 1);
        }
      }
      e += ev;
    }
    tr.e_single = e;
    tr.srfe = do_rf ? sj : 0.0;
    tr.reff = do_rf ? rj : 0.0;
    tr.rf_in = do_rf ? 1 : 0;
  }
}

// RFPAR (srfe, reff) of one ion at (x, y, z): the values INTERACT's cross
// term gathers for every other ion (rfpar.f90:356-367); (0, 0) off the map.
// Positions do not move during GRAND, so the GRAND kernel gathers them once
// and keeps them current through insertions and deletions.
__device__ __forceinline__ double2 rf_single(const KP &p, double x, double y, double z,
                                             int itype) {
  if (!in_grid(p.g3, x, y, z)) return make_double2(0.0, 0.0);
  double si, ri, d1[3], d2[3];
  rfpar_gather(p, x, y, z, rfpar_ifir(p, itype), false, si, ri, d1, d2);
  return make_double2(si, ri);
}

// Trial read past L1: within the GRAND kernel another block wrote it.
__device__ __forceinline__ Trial load_trial_cg(const Trial *t) {
  Trial r;
  const uint2 *src = reinterpret_cast<const uint2 *>(t);
  uint2 *dst = reinterpret_cast<uint2 *>(&r);
#pragma unroll
  for (int k = 0; k < (int)(sizeof(Trial) / sizeof(uint2)); ++k) dst[k] = __ldcg(src + k);
  return r;
}

// What interact_one reads of particle i: position, type and its RFPAR
// (srfe, reff).  Read past L1 (__ldcg): inside the GRAND kernel they change
// between attempts.
struct PartRec {
  double x, y, z;
  double2 rf;
  int ti;
};

// Position of particle i: the FP64 arrays, or (ff, FP32 mode) the
// float-float records as hi + lo in FP64, the value the records stand for.
// Read past L1.
__device__ __forceinline__ double3 pos_of(const KP &p, bool ff, int i) {
  if (ff) {
    const float4 h = __ldcg(p.pk1 + i), l = __ldcg(p.pk2 + i);
    return make_double3((double)h.x + (double)l.x, (double)h.y + (double)l.y,
                        (double)h.z + (double)l.z);
  }
  return make_double3(__ldcg(p.x + i), __ldcg(p.y + i), __ldcg(p.z + i));
}

__device__ __forceinline__ PartRec load_part(const KP &p, int i, bool rf, bool ff = false) {
  PartRec r;
  r.ti = __ldcg(p.typei + i);
  const double3 q = pos_of(p, ff, i);
  r.x = q.x;
  r.y = q.y;
  r.z = q.z;
  r.rf = rf && i >= p.nsites ? __ldcg(p.gc_rf + i) : make_double2(0.0, 0.0);
  return r;
}

// ΔE term of particle i (pair law + RFPAR cross) against the trial, the
// O(N) part of INTERACT; q: the particle's record (load_part).
__device__ double interact_rec(const KP &p, const Trial &tr, uint32_t mask, int i, int jt2,
                               bool beion, bool rf, const PartRec &q, int &err) {
  const bool ion_i = i >= p.nsites;
  const int ti = q.ti;
  if (ion_i && guard_bad(p.st, abs(ti) - p.nold - 1, p.ntype - p.nold, 31)) return 0.0;
  double dx = q.x - tr.x, dy = q.y - tr.y, dz = q.z - tr.z;
  if (p.periodic) {  // extension mode: nearest image, plain cutoff
    dx -= p.lx * rint(dx / p.lx);
    dy -= p.ly * rint(dy / p.ly);
    dz -= p.lz * rint(dz / p.lz);
  }
  const double d2 = dx * dx + dy * dy + dz * dz;
  if (p.periodic && d2 >= p.rc2) return 0.0;
  double u = 0.0;
  if (mask & 1u) {
    int is = -1;
    if (beion && ion_i)  // interact.f90:173-210
      is = p.pidx[(p.nwtype[abs(ti)] - 1) * p.nttyp + jt2 - 1];
    else if (beion && !ion_i)  // interact.f90:351-381
      is = p.pidx[(p.typtyp[i] - 1) * p.nttyp + jt2 - 1];
    else if (!beion && ion_i)  // interact.f90:383-413
      is = p.pidx[(p.nwtype[abs(ti)] - 1) * p.nttyp + jt2 - 1];
    if (is >= 0) u += law_interact64(p, p.pp[is], d2, err);
  }
  if (rf && ion_i) {
    const double2 g = q.rf;
    if (g.x != 0.0) {
      const double tau = p.celec * p.cg[tr.itype];
      const double reffij = tr.reff * g.y;
      u += tau * p.cg[abs(ti)] * reffij * tr.srfe * g.x / sqrt(reffij * reffij + d2);
    }
  }
  return u;
}

__device__ double interact_one(const KP &p, const Trial &tr, uint32_t mask, int i, int jt2,
                               bool beion, bool rf, int &err, bool ff = false) {
  return interact_rec(p, tr, mask, i, jt2, beion, rf, load_part(p, i, rf, ff), err);
}

// Combined type of the trial particle, 0 (and a guard record) when invalid.
__device__ __forceinline__ int trial_type2(const KP &p, const Trial &tr) {
  const int j0 = tr.j - 1;
  if (!tr.valid || guard_bad(p.st, j0, (long long)p.cap + 1, 29)) return 0;
  const int jt2 = j0 >= p.nsites ? p.nwtype[tr.itype] : p.typtyp[j0];
  return guard_bad(p.st, jt2 - 1, p.nttyp, 30) ? 0 : jt2;
}

// RFPAR prepass of INTERACT: (srfe, reff) of every ion at its position.
__global__ void k_rf_prepass(KP p) {
  const int i = p.nsites + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.st->ntot) return;
  p.gc_rf[i] = rf_single(p, p.x[i], p.y[i], p.z[i], abs(p.typei[i]));
}

// Partial ΔE over the other particles, one thread per particle.
__global__ void __launch_bounds__(kIaThreads) k_interact_part(KP p, uint32_t mask) {
  __shared__ double red[kIaThreads / 32];
  __shared__ double tot[1];
  const Trial tr = *p.trial;
  const int ntot = p.st->ntot;
  const int jt2 = trial_type2(p, tr);
  const bool beion = tr.valid && tr.j - 1 >= p.nsites;
  const bool rf = tr.valid && tr.rf_in && (mask & 16u);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double u = 0.0;
  int err = 0;
  if (jt2 > 0 && i < ntot && i != tr.j - 1) u = interact_one(p, tr, mask, i, jt2, beion, rf, err);
  if (err) atomicOr(&p.st->err, err);
  block_sum<1>(&u, red, tot);
  if (threadIdx.x == 0) p.ipart[blockIdx.x] = tot[0];
}

// Sum of the partials plus the trial's single-particle part: the full ΔE.
__device__ double interact_total(const KP &p, const Trial &tr, int nblk, double *red,
                                 double *tot) {
  double v = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) v += __ldcg(p.ipart + b);
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
  if ((mask & 16u) && p.qrfpar && ntot_ub > p.nsites)
    k_rf_prepass<<<(ntot_ub - p.nsites + 127) / 128, 128, 0, stream>>>(p);
  k_interact_prep<<<1, 32, 0, stream>>>(p, mask, qalert);
  k_interact_part<<<nb, kIaThreads, 0, stream>>>(p, mask);
  k_interact_final<<<1, kIaThreads, 0, stream>>>(p, nb, dener_dev);
}

// ---------------------------------------------------------------------------
// GRAND (grand.f90:19-121, insert.f90, find.f90): every attempt of one call
// in one cooperative launch, settled in order, evaluated in rounds.
//
// On this part a warp issues one FP64 instruction per ~64 clocks however
// many of its lanes are active, so an attempt's O(N) ΔE sum costs the FP64
// chain of one pair term whatever the lanes do.  A round therefore
// evaluates the pair terms of every particle against up to kSpec attempts
// at once (lane = particle x attempt), all in the state at the start of
// the round, and block 0 then settles the attempts in order:
//   - up to the round's first acceptance the state is the round's, and the
//     round's sums are those of the sequential algorithm;
//   - after an acceptance, an insertion trial's ΔE is its sum plus its pair
//     terms with the ions the round inserted, minus those with the ions the
//     round deleted (trial-trial terms, formed while the other blocks sum);
//   - a deletion trial keeps its target and sum when the rank drawn from
//     the buffer's current count is the rank the target was found at and
//     no deletion of the round touched the buffer (neither the deleted ion
//     nor the last ion moved into the freed slot belongs to it): ranks of a
//     buffer's ions change only then, an insertion appends its ion last.
//     Otherwise the round ends before that attempt and the next round
//     proposes from the current state.
// The draws, the proposals and their outcomes are those of proposing each
// attempt after the previous one is settled; ΔE agrees to FP64 rounding (a
// correction adds a pair term outside the block partial sums).  Error flags
// of the pair terms and a deletion trial's warnings count only for the
// attempts settled with them.
//
// Per round:
//   block 0: the trials: draws (a thread per attempt), deletion targets in
//            the current state (one block scan for all), single-particle
//            terms (a warp per trial); publish the round (release bar_gen);
//   blocks 1..: pair terms, lane = (particle, attempt) -> per-block partial
//            of each attempt (ipart) and its error flags (ierr); arrive on
//            bar_count (release);
//   block 0, meanwhile: each trial's particle as an ion record holds it
//            (with its RFPAR srfe, reff) and the trial-trial pair terms; after
//            every arrival (acquire) the totals, the acceptances of all
//            attempts as if none before them were accepted (in parallel),
//            then the settling in order.
// A round with no attempts ends the launch.  Each thread owns the same
// particles in every round and keeps its first particle's record across
// rounds, re-read only when the round header names the slot as rewritten.
// Data another block wrote during the launch are read past L1 (__ldcg).
// Every wait is bounded: it gives up after kWaitSpins polls, or as soon as
// another block has given up, records kErrBarrier and the launch returns.
// ---------------------------------------------------------------------------
constexpr int kGrandThreads = 128;
constexpr int kGrandWarps = kGrandThreads / 32;

// Lanes per particle in the pair phase: the attempts of a round rounded up
// to a power of two (lane = particle * lanes + attempt).
__host__ __device__ inline int grand_lanes(int ngcmc) {
  const int a = ngcmc < 1 ? 1 : (ngcmc < kSpec ? ngcmc : kSpec);
  int ap = 1;
  while (ap < a) ap <<= 1;
  return ap;
}

struct GrandState {
  Trial tr[kSpec];          // the round's trials
  double u_rank[kSpec];     // deletion: the rank draw
  double u_acc[kSpec];      // the acceptance draw
  int ip0[kSpec];           // deletion: the rank its target was found at, 0 none
  int need[kSpec], found[kSpec];
  int nalert[kSpec];        // deletion: warnings of its single-particle terms
  // each trial's particle as an ion record holds it: position (float-float
  // rounded in FP32 mode), signed type, RFPAR (srfe, reff) at that position
  double px[kSpec], py[kSpec], pz[kSpec];
  double2 rf[kSpec];
  int ti[kSpec];
  double tt[kSpec][kSpec];  // tt[k][a], k < a: trial a's pair term with k's particle
  int terr[kSpec][kSpec];
  double base[kSpec];       // the round's sums, totalled over the blocks
  int aerr[kSpec];
  double de0[kSpec];        // ΔE and acceptance with no acceptance earlier
  int acc0[kSpec];          // in the round
  int pbuf[kSpec], pdel[kSpec];  // buffer (0-based) whose count the attempt changed, by
  int nat0[kMaxBuffers];    // the buffer counts at the start of the round
  int scan[kGrandWarps][kSpec];
  int nchg, chg[kSpec];     // slots the last round rewrote
  int done;                 // attempts the round settled
  int ntot, ff, nbuf;
  int nat[kMaxBuffers], ninsert[kMaxBuffers], nremove[kMaxBuffers], ntotat[kMaxBuffers];
  double dener_sum;
  // buffer parameters, 1-based as in KP
  double avnum[kMaxBuffers + 1], mu[kMaxBuffers + 1], kbb[kMaxBuffers + 1];
  double lzmin[kMaxBuffers + 1], lzmax[kMaxBuffers + 1];
  double rmin[kMaxBuffers + 1], rmax[kMaxBuffers + 1];
  int ibfftyp[kMaxBuffers + 1], qbias[kMaxBuffers + 1];
};

// The attempt's uniform draws, gcmc_uniform(seed, cycle, attempt, n) for
// n = 0, 1, ..., with one Philox block per four draws.
struct Draws {
  uint64_t seed, cycle;
  uint32_t attempt, n = 0, blk = 0xffffffffu;
  uint32_t w[4];
  __device__ double next() {
    if ((n >> 2) != blk) {
      blk = n >> 2;
      philox4x32_10(attempt, blk, (uint32_t)cycle,
                    ((uint32_t)(cycle >> 32) & 0x00FFFFFFu) | (2u << 24), (uint32_t)seed,
                    (uint32_t)(seed >> 32), w);
    }
    return u01(w[n++ & 3]);
  }
};

// The random part of one attempt's proposal (grand.f90:42-86): insertion
// or deletion, the buffer, for an insertion its point by rejection sampling
// inside the buffer (insert.f90), for a deletion the uniform its rank is
// drawn from (find.f90).  None depends on the state.
__device__ void propose_draws(const KP &p, uint64_t seed, uint64_t cycle, uint32_t attempt,
                              const GrandState &g, Trial &t, double &u_rank) {
  t = Trial{};
  Draws d{seed, cycle, attempt};
  const int nbuf = g.nbuf;
  u_rank = 0.0;
  if (d.next() < 0.5) {
    const int ib = (int)((double)nbuf * d.next()) + 1;
    t.insert = 1;
    t.ib = ib;
    if (ib <= nbuf && g.avnum[ib] > 0.0) {
      t.itype = g.ibfftyp[ib];
      t.valid = 1;
      bool ok = false;
      for (int it = 0; it < (1 << 20) && !ok; ++it) {
        const double u1 = d.next(), u2 = d.next(), u3 = d.next();
        t.x = p.lx * (u1 - 0.5) + p.cx;
        t.y = p.ly * (u2 - 0.5) + p.cy;
        t.z = g.lzmin[ib] + (g.lzmax[ib] - g.lzmin[ib]) * u3;
        ok = true;
        if (p.shape == 1) {
          const double r2 = (t.x - p.cx) * (t.x - p.cx) + (t.y - p.cy) * (t.y - p.cy) +
                            (t.z - p.cz) * (t.z - p.cz);
          ok = r2 > g.rmin[ib] * g.rmin[ib] && r2 < g.rmax[ib] * g.rmax[ib];
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
    t.ib = (int)((double)nbuf * d.next()) + 1;
    u_rank = d.next();
    t.insert = 0;
  }
  t.draw = (int)d.n;
}

// find.f90 for every deletion trial k of the round with need[k]: the slot
// of the ip0[k]-th ion of buffer tr[k].ib in slot order into found[k] (left
// at -1 if none).  Block 0, every thread; one pass over the buffer tags.
__device__ void find_ranks(const KP &p, GrandState &g, int na) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int lo = p.nsites + p.nfix, ntot = g.ntot;
  const int per = (ntot - lo + (int)blockDim.x - 1) / (int)blockDim.x;
  const int a = lo + threadIdx.x * per, b = min(ntot, a + per);
  int ib[kSpec], c[kSpec];
#pragma unroll
  for (int k = 0; k < kSpec; ++k) {
    ib[k] = k < na && g.need[k] ? g.tr[k].ib : -1;
    c[k] = 0;
  }
  for (int s = a; s < b; ++s) {
    const int v = p.ibuffer[s];
#pragma unroll
    for (int k = 0; k < kSpec; ++k) c[k] += v == ib[k];
  }
  int before[kSpec];
#pragma unroll
  for (int k = 0; k < kSpec; ++k) {  // inclusive scans: warp shuffles, then warp totals
    int incl = c[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) g.scan[wid][k] = incl;
    before[k] = incl - c[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kSpec; ++k) {
    if (ib[k] < 0) continue;
    for (int w = 0; w < wid; ++w) before[k] += g.scan[w][k];
    const int rank = g.ip0[k];
    if (rank > before[k] && rank <= before[k] + c[k]) {  // exactly one thread
      int r = before[k];
      for (int s = a; s < b; ++s)
        if (p.ibuffer[s] == ib[k] && ++r == rank) {
          g.found[k] = s;
          break;
        }
    }
  }
  __syncthreads();
}

// The round's trials (block 0, every thread): attempts a0 .. a0+na-1
// proposed in the current state, with their single-particle terms
// (deletion trials count their warnings in nalert, insertion trials raise
// none: grand.f90:48,86) and acceptance draws.
__device__ void build_round(const KP &p, uint32_t mask, uint64_t seed, uint64_t cycle, int a0,
                            int na, GrandState &g) {
  const int t = threadIdx.x;
  if (t < na) {
    Trial tr;
    double u = 0.0;
    propose_draws(p, seed, cycle, (uint32_t)(a0 + t), g, tr, u);
    tr.ntot = g.ntot;
    tr.chg = -1;
    g.need[t] = 0;
    g.found[t] = -1;
    g.nalert[t] = 0;
    g.ip0[t] = 0;
    if (tr.insert) {
      tr.j = g.ntot + 1;
    } else {
      const int ib = tr.ib;
      const int natb = ib <= g.nbuf ? g.nat[ib - 1] : 0;
      const int ip = (int)((double)natb * u) + 1;
      tr.valid = 0;
      if (ib <= g.nbuf && ip <= natb) {
        tr.itype = g.ibfftyp[ib];
        tr.valid = 1;
        g.need[t] = 1;
        g.ip0[t] = ip;
      }
    }
    g.tr[t] = tr;
    g.u_rank[t] = u;
    g.u_acc[t] = gcmc_uniform(seed, cycle, (uint32_t)(a0 + t), (uint32_t)tr.draw);
  }
  __syncthreads();
  find_ranks(p, g, na);
  if (t < na && g.need[t]) {
    Trial &tr = g.tr[t];
    const int k = g.found[t];
    if (k < 0 || guard_bad(p.st, k, g.ntot, 11)) {
      tr.valid = 0;
      g.ip0[t] = 0;
      atomicOr(&p.st->err, kErrFind);
    } else {
      tr.j = k + 1;
      const double3 q = pos_of(p, g.ff, k);
      tr.x = q.x;
      tr.y = q.y;
      tr.z = q.z;
    }
  }
  __syncthreads();
  for (int k = t >> 5; k < na; k += kGrandWarps) {
    Trial tr = g.tr[k];
    if (tr.valid) {
      trial_single_warp(p, tr, mask, tr.insert ? 0 : 1, &g.nalert[k]);
      if ((t & 31) == 0) {
        g.tr[k].e_single = tr.e_single;
        g.tr[k].srfe = tr.srfe;
        g.tr[k].reff = tr.reff;
        g.tr[k].rf_in = tr.rf_in;
      }
    }
  }
  __syncthreads();
}

// A coordinate as its float-float record stores it (hi = fl(x), lo =
// fl(x - hi)), read back as hi + lo.
__device__ __forceinline__ double ff_rounded(double x) {
  const float h = (float)x;
  return (double)h + (double)(float)(x - (double)h);
}

// Each trial's particle as an ion record holds it (block 0, a thread per
// trial): an insertion's what its acceptance writes (the point, rounded to
// the float-float record in FP32 mode; the signed type; RFPAR at the
// record's point), a deletion's its target's record.
__device__ void trial_ions(const KP &p, uint32_t mask, int na, GrandState &g) {
  const int t = threadIdx.x;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  if (t < na) {
    const Trial &tr = g.tr[t];
    double x = tr.x, y = tr.y, z = tr.z;
    int ti = 0;
    double2 rf = make_double2(0.0, 0.0);
    if (tr.valid) {
      if (tr.insert) {
        if (g.ff) {
          x = ff_rounded(x);
          y = ff_rounded(y);
          z = ff_rounded(z);
        }
        ti = tr.z < p.cz ? -tr.itype : tr.itype;
      } else {
        ti = p.typei[tr.j - 1];
      }
      if (rf_on) rf = rf_single(p, x, y, z, abs(ti));
    }
    g.px[t] = x;
    g.py[t] = y;
    g.pz[t] = z;
    g.ti[t] = ti;
    g.rf[t] = rf;
  }
}

// Trial-trial pair terms (block 0, a thread per pair k < a): trial a's
// INTERACT term with trial k's particle as an ion record holds it.
__device__ void trial_pairs(const KP &p, uint32_t mask, int na, GrandState &g) {
  for (int idx = threadIdx.x; idx < na * na; idx += blockDim.x) {
    const int k = idx / na, a = idx - k * na;
    if (k >= a) continue;
    const Trial &ta = g.tr[a], &tk = g.tr[k];
    double v = 0.0;
    int err = 0;
    // two deletions of one ion are never both settled (the first touches
    // the buffer of the second)
    if (ta.valid && tk.valid && (ta.insert || tk.insert || ta.j != tk.j)) {
      const int jt2 = trial_type2(p, ta);
      if (jt2 > 0) {
        PartRec q;
        q.x = g.px[k];
        q.y = g.py[k];
        q.z = g.pz[k];
        q.rf = g.rf[k];
        q.ti = g.ti[k];
        v = interact_rec(p, ta, mask, p.nsites, jt2, true, ta.rf_in && (mask & 16u), q, err);
      }
    }
    g.tt[k][a] = v;
    g.terr[k][a] = err;
  }
}

// Totals of the round's block partials (block 0): warp w for attempts w,
// w + kGrandWarps, ...; a fixed summation order.
__device__ void round_sums(const KP &p, int na, GrandState &g) {
  const int lane = threadIdx.x & 31, nblk = gridDim.x;
  for (int a = threadIdx.x >> 5; a < na; a += kGrandWarps) {
    double v = 0.0;
    int e = 0;
    for (int b = 1 + lane; b < nblk; b += 32) {
      v += __ldcg(p.ipart + (size_t)b * kSpec + a);
      e |= __ldcg(p.ierr + (size_t)b * kSpec + a);
    }
    v = wsum(v);
    e = __reduce_or_sync(0xffffffffu, e);
    if (lane == 0) {
      g.base[a] = v;
      g.aerr[a] = e;
    }
  }
}

// Im-Roux acceptance probability of trial tr with total ΔE de in the
// current state (grand.f90:88-116).
__device__ double accept_rate(const KP &p, const GrandState &g, const Trial &tr, double de,
                              uint64_t cycle) {
  const int ib = tr.ib, b = ib - 1;
  const int nat = g.nat[b];
  const double boltz = exp(-(de - g.mu[ib]) * p.ikbt);
  double rate;
  if (tr.insert) {
    if (g.qbias[ib]) {
      rate = g.avnum[ib] + g.kbb[ib] * (g.avnum[ib] - (double)(g.ntotat[b] / (long long)cycle));
      rate = rate * boltz / (double)(nat + 1);
    } else {
      rate = (g.avnum[ib] / (nat + 1)) * boltz;
    }
    return rate / (1.0 + rate);
  }
  if (g.qbias[ib]) {
    rate = g.avnum[ib] + g.kbb[ib] * (g.avnum[ib] - (double)(g.ntotat[b] / (long long)cycle));
    rate = rate * boltz / (double)nat;
  } else {
    rate = (g.avnum[ib] / nat) * boltz;
  }
  return 1.0 / (1.0 + rate);
}

// ΔE and acceptance of every attempt as if no attempt before it in the
// round were accepted (block 0, a thread per attempt): exact up to the
// round's first acceptance.
__device__ void first_acceptances(const KP &p, uint64_t cycle, int na, GrandState &g) {
  const int a = threadIdx.x;
  if (a >= na) return;
  const Trial &tr = g.tr[a];
  g.de0[a] = 0.0;
  g.acc0[a] = 0;
  if (tr.valid && tr.ib >= 1 && tr.ib <= g.nbuf) {
    const double de = tr.e_single + g.base[a];
    g.de0[a] = de;
    g.acc0[a] = g.u_acc[a] <= accept_rate(p, g, tr, de, cycle);
  }
}

// The round's attempts in order (block 0, thread 0): ΔE, acceptance and the
// insertion or deletion (grand.f90:48-116), until an attempt whose trial no
// longer holds.  g.done: the attempts settled; g.chg: the slots rewritten.
__device__ void settle(const KP &p, uint32_t mask, uint64_t cycle, int na, GrandState &g) {
  const bool rf_on = (mask & 16u) && p.qrfpar;
  bool changed = false;
  unsigned long long touched = 0;  // bit b: an accepted deletion touched buffer b + 1
  int nacc = 0, acc_k[kSpec];
  double acc_s[kSpec];
  int done = 0;
  g.nchg = 0;
  for (int a = 0; a < na; ++a) {
    Trial tr = g.tr[a];
    if (changed && !tr.insert) {  // the deletion trial in the current state
      const int ib = tr.ib;
      const int natb = ib <= g.nbuf ? g.nat[ib - 1] : 0;
      const int ip = (int)((double)natb * g.u_rank[a]) + 1;
      if (!(ib <= g.nbuf && ip <= natb))
        tr.valid = 0;  // no ion left to delete: the attempt does nothing
      else if (g.ip0[a] == 0 || ip != g.ip0[a] || ((touched >> (ib - 1)) & 1ull))
        break;  // another target: propose it again in the next round
    }
    g.pbuf[a] = -1;
    g.pdel[a] = 0;
    int err = 0;
    if (tr.valid && !guard_bad(p.st, tr.ib - 1, p.nbuffer, 21)) {
      const int ib = tr.ib, b = ib - 1;
      double de;
      bool yes;
      err = g.aerr[a];
      if (!changed) {
        de = g.de0[a];
        yes = g.acc0[a] != 0;
      } else {
        double c = 0.0;
        for (int m = 0; m < nacc; ++m) {
          c += acc_s[m] * g.tt[acc_k[m]][a];
          err |= g.terr[acc_k[m]][a];
        }
        de = tr.e_single + g.base[a] + c;
        yes = g.u_acc[a] <= accept_rate(p, g, tr, de, cycle);
      }
      if (!tr.insert && g.nalert[a] > 0) atomicAdd(&p.warn[p.nwtype[tr.itype]], g.nalert[a]);
      if (yes) {
        const int ntot = g.ntot, nat = g.nat[b];
        if (tr.insert) {
          if (ntot + 1 > p.cap) {
            atomicOr(&p.st->err, kErrCapacity);
          } else if (!guard_bad(p.st, ntot, p.cap, 22)) {
            g.dener_sum += de;
            g.nat[b] = nat + 1;
            if (g.ff) {  // the records as k_pack forms them (a mobile ion)
              const float xh = (float)tr.x, yh = (float)tr.y, zh = (float)tr.z;
              const int code = (p.nwtype[tr.itype] - 1) | (1 << 16);
              p.pk1[ntot] = make_float4(xh, yh, zh, __int_as_float(code));
              p.pk2[ntot] = make_float4((float)(tr.x - (double)xh), (float)(tr.y - (double)yh),
                                        (float)(tr.z - (double)zh), 0.0f);
              p.pk3[ntot] =
                  make_float4(0.0f, (float)p.cg[tr.itype], __int_as_float(1 << 1), 0.0f);
            } else {
              p.x[ntot] = tr.x;
              p.y[ntot] = tr.y;
              p.z[ntot] = tr.z;
            }
            p.typei[ntot] = g.ti[a];
            p.ibuffer[ntot] = ib;
            if (rf_on) p.gc_rf[ntot] = g.rf[a];
            g.ntot = ntot + 1;
            g.ninsert[b] += 1;
            g.chg[g.nchg++] = ntot;
            g.pbuf[a] = b;
            g.pdel[a] = 1;
            acc_k[nacc] = a;
            acc_s[nacc++] = 1.0;
            changed = true;
          }
        } else if (!guard_bad(p.st, tr.j - 1, ntot, 23) &&
                   !guard_bad(p.st, ntot - 1, p.cap, 24)) {
          const int iat = tr.j - 1, last = ntot - 1;
          const int bz = p.ibuffer[last];  // the ion the freed slot receives
          g.dener_sum -= de;
          g.nremove[b] += 1;
          if (g.ff) {
            p.pk1[iat] = __ldcg(p.pk1 + last);
            p.pk2[iat] = __ldcg(p.pk2 + last);
            p.pk3[iat] = __ldcg(p.pk3 + last);
          } else {
            p.x[iat] = p.x[last];
            p.y[iat] = p.y[last];
            p.z[iat] = p.z[last];
          }
          p.typei[iat] = p.typei[last];
          p.ibuffer[iat] = bz;
          if (rf_on) p.gc_rf[iat] = __ldcg(p.gc_rf + last);
          g.nat[b] = nat - 1;
          g.ntot = ntot - 1;
          g.chg[g.nchg++] = iat;
          g.pbuf[a] = b;
          g.pdel[a] = -1;
          touched |= 1ull << b;
          if (bz >= 1 && bz <= kMaxBuffers) touched |= 1ull << (bz - 1);
          acc_k[nacc] = a;
          acc_s[nacc++] = -1.0;
          changed = true;
        }
      }
    }
    if (err) atomicOr(&p.st->err, err);
    done = a + 1;
  }
  g.done = done;
}

// prob(ib, nat(ib)) += 1 after each settled attempt (grand.f90:117-119),
// a thread per buffer replaying the round's count changes.
__device__ void round_histogram(const KP &p, GrandState &g) {
  for (int b = threadIdx.x; b < g.nbuf; b += blockDim.x) {
    int n = g.nat0[b];
    for (int a = 0; a < g.done; ++a) {
      if (g.pbuf[a] == b) n += g.pdel[a];
      if (!guard_bad(p.st, n, p.cap + 1, 25)) atomicAdd(&p.prob[(size_t)b * (p.cap + 1) + n], 1);
    }
  }
}

__global__ void __launch_bounds__(kGrandThreads)
    k_grand(KP p, uint32_t mask, uint64_t seed, uint64_t cycle, int ngcmc, int ffpos) {
  __shared__ GrandState g;
  __shared__ double red[kGrandWarps * kSpec];
  __shared__ int ered[kGrandWarps * kSpec];
  __shared__ int flag;
  DevState *st = p.st;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  const int ntot0 = st->ntot;
  bool ok = true;
  if (blockIdx.x == 0) {  // the coordinator: GCMC state into shared memory
    const int nb = p.nbuffer;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      g.nat[b] = st->nat[b];
      g.ninsert[b] = st->ninsert[b];
      g.nremove[b] = st->nremove[b];
      g.ntotat[b] = st->ntotat[b];
    }
    for (int ib = threadIdx.x; ib <= nb; ib += blockDim.x) {
      g.avnum[ib] = p.avnum[ib];
      g.mu[ib] = p.mu[ib];
      g.kbb[ib] = p.kbb[ib];
      g.lzmin[ib] = p.lzmin[ib];
      g.lzmax[ib] = p.lzmax[ib];
      g.rmin[ib] = p.rmin[ib];
      g.rmax[ib] = p.rmax[ib];
      g.ibfftyp[ib] = p.ibfftyp[ib];
      g.qbias[ib] = p.qbufferbias[ib];
    }
    if (threadIdx.x == 0) {
      g.ntot = ntot0;
      g.dener_sum = st->dener_sum;
      g.ff = ffpos;
      g.nbuf = nb;
      g.nchg = 0;
    }
    __syncthreads();
    int a0 = 0;
    for (unsigned r = 1; ok; ++r) {
      const int na = min(ngcmc - a0, kSpec);
      if (na > 0) build_round(p, mask, seed, cycle, a0, na, g);
      if (threadIdx.x == 0) {  // publish the round
        GrandRound *hd = p.ground;
        hd->a0 = a0;
        hd->na = na;
        hd->ntot = g.ntot;
        hd->nchg = g.nchg;
        for (int c = 0; c < g.nchg; ++c) hd->chg[c] = g.chg[c];
        for (int k = 0; k < na; ++k) p.trial[k] = g.tr[k];
        __threadfence();
        release_add(&st->bar_gen, 1u);
      }
      if (na <= 0) break;
      trial_ions(p, mask, na, g);
      for (int b = threadIdx.x; b < nb; b += blockDim.x) g.nat0[b] = g.nat[b];
      __syncthreads();
      trial_pairs(p, mask, na, g);
      if (!(ok = block_wait(&st->bar_count, (unsigned)(gridDim.x - 1) * r, st, &flag))) break;
      round_sums(p, na, g);
      __syncthreads();
      first_acceptances(p, cycle, na, g);
      __syncthreads();
      if (threadIdx.x == 0) settle(p, mask, cycle, na, g);
      __syncthreads();
      round_histogram(p, g);
      a0 += g.done;
      __syncthreads();
    }
    // GCMC state back to the device record (also after a failed wait)
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
      st->nat[b] = g.nat[b];
      st->ninsert[b] = g.ninsert[b];
      st->nremove[b] = g.nremove[b];
    }
    if (threadIdx.x == 0) {
      st->ntot = g.ntot;
      st->dener_sum = g.dener_sum;
    }
    return;
  }
  // blocks 1..: the pair terms.  Warp wg of the pair phase holds particles
  // wg * per_warp + lane / ap, then + stride, ...; lane & (ap - 1) is the
  // lane's attempt within the round.
  const int ap = grand_lanes(ngcmc), per_warp = 32 / ap;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, la = lane & (ap - 1);
  const int stride = (gridDim.x - 1) * kGrandWarps * per_warp;
  const int i0 = ((blockIdx.x - 1) * kGrandWarps + wid) * per_warp + lane / ap;
  // RFPAR prepass: one lane per particle, at its position; the first
  // particle's record (its RFPAR from that lane) is kept across rounds
  double2 rf0 = make_double2(0.0, 0.0);
  if (rf_on && la == 0)
    for (int i = i0; i < ntot0; i += stride)
      if (i >= p.nsites) {
        const double3 q = pos_of(p, ffpos, i);
        const double2 v = rf_single(p, q.x, q.y, q.z, abs(p.typei[i]));
        p.gc_rf[i] = v;
        if (i == i0) rf0 = v;
      }
  PartRec pre{};
  if (i0 < ntot0) pre = load_part(p, i0, false, ffpos);
  pre.rf.x = __shfl_sync(0xffffffffu, rf0.x, lane & ~(ap - 1));
  pre.rf.y = __shfl_sync(0xffffffffu, rf0.y, lane & ~(ap - 1));
  for (unsigned r = 1; ok; ++r) {
    if (!(ok = block_wait(&st->bar_gen, r, st, &flag))) break;
    const GrandRound *hd = p.ground;
    const int na = __ldcg(&hd->na);
    if (na <= 0) break;
    const int ntot = __ldcg(&hd->ntot), nchg = __ldcg(&hd->nchg);
    for (int c = 0; c < nchg; ++c)  // the previous round rewrote this slot
      if (__ldcg(&hd->chg[c]) == i0 && i0 < ntot) pre = load_part(p, i0, rf_on, ffpos);
    Trial tr{};
    if (la < na) tr = load_trial_cg(p.trial + la);
    const int jt2 = trial_type2(p, tr);
    const bool beion = tr.valid && tr.j - 1 >= p.nsites;
    const bool rf = tr.valid && tr.rf_in && (mask & 16u);
    double u = 0.0;
    int err = 0;
    if (jt2 > 0)
      for (int i = i0; i < ntot; i += stride)
        if (i != tr.j - 1)
          u += i == i0 ? interact_rec(p, tr, mask, i, jt2, beion, rf, pre, err)
                       : interact_one(p, tr, mask, i, jt2, beion, rf, err, ffpos);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      if (o >= ap) {  // lanes of one attempt
        u += __shfl_xor_sync(0xffffffffu, u, o);
        err |= __shfl_xor_sync(0xffffffffu, err, o);
      }
    if (lane < ap) {
      red[wid * kSpec + lane] = u;
      ered[wid * kSpec + lane] = err;
    }
    __syncthreads();
    if (threadIdx.x < na) {
      double s = 0.0;
      int e = 0;
      for (int w = 0; w < kGrandWarps; ++w) {
        s += red[w * kSpec + threadIdx.x];
        e |= ered[w * kSpec + threadIdx.x];
      }
      p.ipart[(size_t)blockIdx.x * kSpec + threadIdx.x] = s;
      p.ierr[(size_t)blockIdx.x * kSpec + threadIdx.x] = e;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      release_add(&st->bar_count, 1u);
    }
  }
}

// Blocks of the GRAND launch: the coordinator and enough blocks for a lane
// per (particle, attempt of a round), all co-resident, at most the partial
// slots the context holds (ipart_slots); with fewer, a lane takes several
// particles.
cudaError_t launch_grand(const KP &p, int ntot_ub, int ipart_slots, uint32_t mask,
                         uint64_t seed, uint64_t cycle, int ngcmc, int ffpos,
                         cudaStream_t stream) {
  static int max_res[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (max_res[dev] == 0) {
    int per_sm = 0, nsm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_grand, kGrandThreads,
                                                           0)) != cudaSuccess)
      return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return e;
    max_res[dev] = std::max(2, per_sm * nsm);
  }
  const int per_warp = 32 / grand_lanes(ngcmc);
  const int warps = (ntot_ub + ngcmc + per_warp - 1) / per_warp;
  int grid = (warps + kGrandWarps - 1) / kGrandWarps + 1;  // + block 0, the coordinator
  grid = std::max(2, std::min(std::min(grid, max_res[dev]), ipart_slots));
  // both launch counters start at zero
  if ((e = cudaMemsetAsync(&p.st->bar_count, 0, 2 * sizeof(unsigned), stream)) != cudaSuccess)
    return e;
  KP pc = p;
  void *args[] = {(void *)&pc, (void *)&mask, (void *)&seed, (void *)&cycle, (void *)&ngcmc,
                  (void *)&ffpos};
  return cudaLaunchCooperativeKernel((const void *)k_grand, dim3(grid), dim3(kGrandThreads),
                                     args, 0, stream);
}

}  // namespace bgpu
