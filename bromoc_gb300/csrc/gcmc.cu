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
// in one cooperative launch.  Block 0 owns the GCMC state (live count,
// buffer counters, buffer parameters) in shared memory for the whole launch
// and writes it back at the end; the other blocks only sum ΔE.  Per attempt:
//   block 0: the proposal and the trial's single-particle terms; publish
//            the trial (generation flag, release);
//   every block: its share of the O(N) ΔE sum -> ipart[block]; arrive on a
//            counter (release);
//   block 0: while the other blocks sum, the next attempt's random draws
//            (they do not depend on the outcome) and, for an insertion, the
//            next trial's single-particle terms (they depend only on its
//            position); then waits for every arrival (acquire), total ΔE,
//            Im-Roux acceptance, insertion/deletion, counters, and the part
//            of the next proposal that depends on the new state (the live
//            count; for a deletion the rank of its ion, which slot holds it
//            and its single-particle terms).
// One synchronisation per attempt.  Each thread owns the same particles in
// every phase (round-robin over blocks): it reads its particle's record
// before waiting for the next trial, and re-reads it only if the trial
// names its slot as the one the last accepted move rewrote.  Block 0
// proposes the first attempt before its share of the RFPAR prepass.  Data
// that another block wrote during the launch are read past L1 (__ldcg).
// With more than one block, block 0 owns no particles.  In FP32 mode
// (ffpos) the positions are read from and written to the float-float
// records, so no conversion kernel runs around the call.
// Every wait is bounded: it gives up after kWaitSpins polls, or as soon as
// another block has given up, records kErrBarrier and the launch returns.
// The draws, the proposals and their outcomes are those of proposing
// each attempt after the previous one is settled.
// ---------------------------------------------------------------------------
constexpr int kGrandThreads = 128;

struct GrandState {
  Trial s;                  // current trial
  double2 trial_rf;         // RFPAR (srfe, reff) at an insertion trial
  Trial nx;                 // the next attempt's draws (+ insertion terms)
  double nx_u;              // the next deletion's rank draw
  double2 nx_rf;            // RFPAR (srfe, reff) of the next insertion trial
  int nx_fields;            // nx holds the trial's single-particle terms (an
                            // insertion's, or a deletion's found in the state
                            // before the pending acceptance)
  int nx_alert;             // warnings of that deletion trial, not yet counted
  int chg;                  // slot the last accepted move rewrote, -1 none
  int ff;                   // FP32 mode: positions live in the float-float records
  int ntot;
  int nat[kMaxBuffers], ninsert[kMaxBuffers], nremove[kMaxBuffers], ntotat[kMaxBuffers];
  double dener_sum;
  // buffer parameters, 1-based as in KP
  double avnum[kMaxBuffers + 1], mu[kMaxBuffers + 1], kbb[kMaxBuffers + 1];
  double lzmin[kMaxBuffers + 1], lzmax[kMaxBuffers + 1];
  double rmin[kMaxBuffers + 1], rmax[kMaxBuffers + 1];
  int ibfftyp[kMaxBuffers + 1], qbias[kMaxBuffers + 1];
  int scan[kGrandThreads / 32];
  int found;
  double red[kGrandThreads / 32], tot[1];
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

// The random part of one attempt's proposal (grand.f90:42-86), thread 0 of
// block 0: insertion or deletion, the buffer, for an insertion its point by
// rejection sampling inside the buffer (insert.f90), for a deletion the
// uniform its rank is drawn from (find.f90).  None depends on the state.
__device__ void propose_draws(const KP &p, uint64_t seed, uint64_t cycle, uint32_t attempt,
                              GrandState &g) {
  Trial t{};
  Draws d{seed, cycle, attempt};
  const int nbuf = p.nbuffer;
  double u_rank = 0.0;
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
  g.nx = t;
  g.nx_u = u_rank;
  g.nx_fields = 0;
}

// find.f90: the slot of the rank-th ion of buffer ib in slot order, -1 if
// none; block 0, every thread, result in g.found.
__device__ void find_rank(const KP &p, GrandState &g, int ib, int rank) {
  __syncthreads();
  if (threadIdx.x == 0) g.found = -1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int lo = p.nsites + p.nfix, ntot = g.ntot;
  const int per = (ntot - lo + (int)blockDim.x - 1) / (int)blockDim.x;
  const int a = lo + threadIdx.x * per, b = min(ntot, a + per);
  int c = 0;
  for (int k = a; k < b; ++k) c += (p.ibuffer[k] == ib);
  int incl = c;  // inclusive scan: warp shuffles, then the warp totals
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) g.scan[wid] = incl;
  __syncthreads();
  int before = incl - c;
  for (int w = 0; w < wid; ++w) before += g.scan[w];
  if (rank > before && rank <= before + c) {  // exactly one thread
    int r = before;
    for (int k = a; k < b; ++k)
      if (p.ibuffer[k] == ib && ++r == rank) {
        g.found = k;
        break;
      }
  }
  __syncthreads();
}

// The next trial's single-particle terms ahead of the pending acceptance,
// block 0 (every thread).  An insertion's depend on its point only: warp 0
// its terms, warp 1 its RFPAR (srfe, reff).  A deletion's are found in the
// current state (its rank from the current buffer count, the slot, the
// terms, warnings counted but not yet added): exact if the acceptance
// changes nothing, else redone by propose_finish.
__device__ void next_terms(const KP &p, uint32_t mask, GrandState &g) {
  __syncthreads();
  Trial t = g.nx;
  if (t.insert) {
    if (t.valid) {
      t.j = p.nsites + 1;  // any ion slot: the terms of an ion at t's point
      if (threadIdx.x < 32) {
        trial_single_warp(p, t, mask, 0);
        if (threadIdx.x == 0) {
          g.nx.e_single = t.e_single;
          g.nx.srfe = t.srfe;
          g.nx.reff = t.reff;
          g.nx.rf_in = t.rf_in;
        }
      } else if (threadIdx.x == 32 && (mask & 16u) && p.qrfpar) {
        g.nx_rf = rf_single(p, t.x, t.y, t.z, t.itype);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) g.nx_fields = t.valid;
    return;
  }
  const int nbuf = p.nbuffer, ib = t.ib;
  const int natb = ib <= nbuf ? g.nat[ib - 1] : 0;
  const int ip = (int)((double)natb * g.nx_u) + 1;
  if (!(ib <= nbuf && ip <= natb)) return;  // block-uniform: nothing to find
  find_rank(p, g, ib, ip);
  const int k = g.found;
  if (k < 0 || k >= g.ntot) return;
  t.itype = g.ibfftyp[ib];
  t.valid = 1;
  t.j = k + 1;
  const double3 q = pos_of(p, g.ff, k);
  t.x = q.x;
  t.y = q.y;
  t.z = q.z;
  if (threadIdx.x == 0) g.nx_alert = 0;
  __syncthreads();
  if (threadIdx.x < 32) {
    trial_single_warp(p, t, mask, 1, &g.nx_alert);
    if (threadIdx.x == 0) {
      g.nx = t;
      g.nx_fields = 1;
    }
  }
  __syncthreads();
}

// The state-dependent part of the proposal, block 0: the live count, for a
// deletion the rank-th ion of the buffer in slot order (find.f90) and its
// single-particle terms (deletion trials raise warnings as INTERACT with
// Qalert does, insertion trials do not: grand.f90:48,86); g.nx -> g.s.
// Terms that next_terms found ahead are kept when they still hold: always
// for an insertion, for a deletion when the acceptance changed nothing.
__device__ void propose_finish(const KP &p, uint32_t mask, GrandState &g) {
  __syncthreads();
  const bool keep = g.nx_fields && (g.nx.insert || g.chg < 0);
  if (threadIdx.x == 0) {
    Trial t = g.nx;
    const int ntot = g.ntot, nbuf = p.nbuffer;
    if (t.insert) {
      t.j = ntot + 1;
    } else if (keep) {
      if (g.nx_alert > 0) atomicAdd(&p.warn[p.nwtype[t.itype]], g.nx_alert);
    } else {
      const int ib = t.ib;
      const int natb = ib <= nbuf ? g.nat[ib - 1] : 0;
      const int ip = (int)((double)natb * g.nx_u) + 1;
      t.valid = 0;
      if (ib <= nbuf && ip <= natb) {
        t.itype = g.ibfftyp[ib];
        t.valid = 1;
        t.j = ip;  // rank within the buffer; resolved to a slot below
      }
    }
    t.ntot = ntot;
    t.chg = g.chg;
    g.s = t;
    if (t.insert) g.trial_rf = g.nx_rf;
  }
  __syncthreads();
  if (keep) return;
  const Trial &s = g.s;
  if (s.valid && !s.insert) {
    find_rank(p, g, s.ib, s.j);
    if (threadIdx.x == 0) {
      const int k = g.found;
      if (k < 0 || guard_bad(p.st, k, g.ntot, 11)) {
        g.s.valid = 0;
        atomicOr(&p.st->err, kErrFind);
      } else {
        g.s.j = k + 1;
        const double3 q = pos_of(p, g.ff, k);
        g.s.x = q.x;
        g.s.y = q.y;
        g.s.z = q.z;
      }
    }
    __syncthreads();
    if (threadIdx.x < 32 && g.s.valid) {
      Trial t = g.s;
      trial_single_warp(p, t, mask, 1);
      if (threadIdx.x == 0) g.s = t;
    }
  } else if (s.valid && s.insert) {  // not computed ahead
    if (threadIdx.x < 32) {
      Trial t = g.s;
      trial_single_warp(p, t, mask, 0);
      if (threadIdx.x == 0) g.s = t;
    } else if (threadIdx.x == 32 && (mask & 16u) && p.qrfpar) {
      g.trial_rf = rf_single(p, g.s.x, g.s.y, g.s.z, g.s.itype);
    }
  }
  __syncthreads();
}

// Total ΔE, Im-Roux acceptance and the insertion/deletion (grand.f90:48-116)
// of the current trial; block 0, state in g.  g.chg: the slot an accepted
// move rewrote (the new ion's, or the deleted ion's that the last ion
// fills), -1 otherwise.
__device__ void accept(const KP &p, uint32_t mask, int nblk, uint64_t seed, uint64_t cycle,
                       uint32_t attempt, GrandState &g) {
  const Trial &tr = g.s;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  double dener = 0.0;
  if (tr.valid) dener = interact_total(p, tr, nblk, g.red, g.tot);
  if (threadIdx.x == 0) g.chg = -1;
  if (threadIdx.x == 0 && tr.valid && !guard_bad(p.st, tr.ib - 1, p.nbuffer, 21)) {
    const int ib = tr.ib, b = ib - 1;
    const int nat = g.nat[b];
    const double boltz = exp(-(dener - g.mu[ib]) * p.ikbt);
    double rate;
    if (tr.insert) {
      if (g.qbias[ib]) {
        rate = g.avnum[ib] + g.kbb[ib] * (g.avnum[ib] - (double)(g.ntotat[b] / (long long)cycle));
        rate = rate * boltz / (double)(nat + 1);
      } else {
        rate = (g.avnum[ib] / (nat + 1)) * boltz;
      }
      rate = rate / (1.0 + rate);
    } else {
      if (g.qbias[ib]) {
        rate = g.avnum[ib] + g.kbb[ib] * (g.avnum[ib] - (double)(g.ntotat[b] / (long long)cycle));
        rate = rate * boltz / (double)nat;
      } else {
        rate = (g.avnum[ib] / nat) * boltz;
      }
      rate = 1.0 / (1.0 + rate);
    }
    if (gcmc_uniform(seed, cycle, attempt, (uint32_t)tr.draw) <= rate) {
      const int ntot = g.ntot;
      if (tr.insert) {
        if (ntot + 1 > p.cap) {
          atomicOr(&p.st->err, kErrCapacity);
        } else if (!guard_bad(p.st, ntot, p.cap, 22)) {
          g.dener_sum += dener;
          g.nat[b] = nat + 1;
          if (g.ff) {  // the records as k_pack forms them (a mobile ion)
            const float xh = (float)tr.x, yh = (float)tr.y, zh = (float)tr.z;
            const int code = (p.nwtype[tr.itype] - 1) | (1 << 16);
            p.pk1[ntot] = make_float4(xh, yh, zh, __int_as_float(code));
            p.pk2[ntot] = make_float4((float)(tr.x - (double)xh), (float)(tr.y - (double)yh),
                                      (float)(tr.z - (double)zh), 0.0f);
            p.pk3[ntot] = make_float4(0.0f, (float)p.cg[tr.itype], __int_as_float(1 << 1), 0.0f);
          } else {
            p.x[ntot] = tr.x;
            p.y[ntot] = tr.y;
            p.z[ntot] = tr.z;
          }
          p.typei[ntot] = tr.z < p.cz ? -tr.itype : tr.itype;
          p.ibuffer[ntot] = ib;
          if (rf_on) p.gc_rf[ntot] = g.trial_rf;
          g.ntot = ntot + 1;
          g.ninsert[b] += 1;
          g.chg = ntot;
        }
      } else if (!guard_bad(p.st, tr.j - 1, ntot, 23) &&
                 !guard_bad(p.st, ntot - 1, p.cap, 24)) {
        const int iat = tr.j - 1, last = ntot - 1;
        g.dener_sum -= dener;
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
        p.ibuffer[iat] = p.ibuffer[last];
        if (rf_on) p.gc_rf[iat] = __ldcg(p.gc_rf + last);
        g.nat[b] = nat - 1;
        g.ntot = ntot - 1;
        g.chg = iat;
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < p.nbuffer; b += blockDim.x)  // prob(ib, nat(ib)) += 1
    if (!guard_bad(p.st, g.nat[b], p.cap + 1, 25))
      atomicAdd(&p.prob[(size_t)b * (p.cap + 1) + g.nat[b]], 1);
}

__global__ void __launch_bounds__(kGrandThreads)
    k_grand(KP p, uint32_t mask, uint64_t seed, uint64_t cycle, int ngcmc, int ffpos) {
  __shared__ GrandState g;
  __shared__ int flag;
  DevState *st = p.st;
  const bool b0 = blockIdx.x == 0;
  // particles round-robin over the blocks; with more than one block, block 0
  // only coordinates (its proposals and acceptances stay off the ΔE sums)
  const int nwb = gridDim.x > 1 ? gridDim.x - 1 : 1;
  const bool owns = gridDim.x == 1 || !b0;
  const int nthr = nwb * blockDim.x;
  const int gtid = owns ? threadIdx.x * nwb + (gridDim.x > 1 ? blockIdx.x - 1 : 0) : nthr;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  const int ntot0 = st->ntot;
  bool ok = true;
  if (b0) {  // GCMC state into shared memory, then the first proposal
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
      g.chg = -1;
      g.ff = ffpos;
    }
    __syncthreads();
    if (ngcmc > 0) {
      if (threadIdx.x == 0) propose_draws(p, seed, cycle, 0u, g);
      propose_finish(p, mask, g);
      if (threadIdx.x == 0) {
        *p.trial = g.s;
        release_add(&st->bar_gen, 1u);
      }
    }
  }
  if (rf_on)  // RFPAR prepass, each thread its own particles
    for (int i = gtid; i < ntot0; i += nthr)
      if (i >= p.nsites) {
        const double3 q = pos_of(p, ffpos, i);
        p.gc_rf[i] = rf_single(p, q.x, q.y, q.z, abs(p.typei[i]));
      }
  // this thread's first particle, read ahead of each attempt
  PartRec pre{};
  if (gtid < ntot0) pre = load_part(p, gtid, rf_on, ffpos);
  for (int a = 0; a < ngcmc && ok; ++a) {
    if (!b0 && !(ok = block_wait(&st->bar_gen, (unsigned)(a + 1), st, &flag))) break;
    const Trial tr = b0 ? g.s : load_trial_cg(p.trial);
    const int jt2 = trial_type2(p, tr);
    const bool beion = tr.valid && tr.j - 1 >= p.nsites;
    const bool rf = tr.valid && tr.rf_in && (mask & 16u);
    if (gtid == tr.chg) pre = load_part(p, gtid, rf_on, ffpos);  // rewritten by the last move
    double u = 0.0;
    int err = 0;
    if (jt2 > 0)
      for (int i = gtid; i < tr.ntot; i += nthr)
        if (i != tr.j - 1)
          u += i == gtid ? interact_rec(p, tr, mask, i, jt2, beion, rf, pre, err)
                         : interact_one(p, tr, mask, i, jt2, beion, rf, err, ffpos);
    if (err) atomicOr(&st->err, err);
    double *red = g.red, *tot = g.tot;
    block_sum<1>(&u, red, tot);
    if (threadIdx.x == 0) {
      p.ipart[blockIdx.x] = tot[0];
      release_add(&st->bar_count, 1u);
    }
    if (b0) {
      const bool more = a + 1 < ngcmc;
      if (more) {  // the next attempt's draws (and insertion terms) meanwhile
        if (threadIdx.x == 0) propose_draws(p, seed, cycle, (uint32_t)(a + 1), g);
        next_terms(p, mask, g);
      }
      if (!(ok = block_wait(&st->bar_count, (unsigned)(gridDim.x * (a + 1)), st, &flag))) break;
      accept(p, mask, gridDim.x, seed, cycle, (uint32_t)a, g);
      if (more) {
        propose_finish(p, mask, g);
        if (threadIdx.x == 0) {
          *p.trial = g.s;
          release_add(&st->bar_gen, 1u);
        }
      }
    }
  }
  if (b0) {  // GCMC state back to the device record (also after a failed wait)
    __syncthreads();
    for (int b = threadIdx.x; b < p.nbuffer; b += blockDim.x) {
      st->nat[b] = g.nat[b];
      st->ninsert[b] = g.ninsert[b];
      st->nremove[b] = g.nremove[b];
    }
    if (threadIdx.x == 0) {
      st->ntot = g.ntot;
      st->dener_sum = g.dener_sum;
    }
  }
}

// Blocks of the GRAND launch: about one per 64 particles, all co-resident,
// at most the ipart slots the context holds (ipart_slots).
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
    max_res[dev] = std::max(1, per_sm * nsm);
  }
  int grid = (ntot_ub + ngcmc + 63) / 64 + 1;  // + block 0, the coordinator
  grid = std::max(1, std::min(std::min(grid, max_res[dev]), ipart_slots));
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
