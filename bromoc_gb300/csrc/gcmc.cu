// INTERACT (interact.f90) and GRAND (grand.f90, insert.f90, find.f90) on the
// device, all in FP64.  INTERACT alone is four launches (RFPAR prepass, the
// trial's single-particle terms, the O(N) sum, the total); GRAND runs all
// its attempts in one cooperative launch (k_grand).  The live particle count
// stays on the device (DevState::ntot).
#include <algorithm>

#include "ffmath.cuh"
#include "gridsync.cuh"
#include "batch.cuh"
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

// INTERACT entry: the trial is written; one warp fills its single part.
// qalert < 0: a deletion trial counts its warnings, an insertion none
// (grand.f90:48,86).  An invalid trial gets no terms.
__global__ void __launch_bounds__(32) k_interact_prep(KP p, uint32_t mask, int qalert) {
  __shared__ Trial s;
  if (threadIdx.x == 0) s = *p.trial;
  __syncwarp();
  Trial t = s;
  if (!t.valid) {
    t.e_single = t.srfe = t.reff = 0.0;
    t.rf_in = 0;
  } else {
    trial_single_warp(p, t, mask, qalert < 0 ? !t.insert : qalert);
  }
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
  if ((mask & 64u) && p.mm.on)  // interact.f90:121-141
    launch_mmij_interact(p, ntot_ub, dener_dev, stream);
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

// ---- tables of the GRAND kernel ---------------------------------------------
// The type and pair-law tables its serial paths read, copied into shared
// memory when they fit (a lookup then costs an SM round trip, not an L2
// one); otherwise the refs point at the global arrays.
constexpr int kShTypes = kMaxTypes + 1, kShPidx = 1024, kShPairs = 48;
struct TypeRefs {
  const int *nwtype, *rfmap, *vmap;
  const float2 *qc, *cg, *esv;
};
struct PairRefs {
  const int *pidx, *nwtype;
  const PairFF *ppff;
};
struct GrandTabs {
  int nwtype[kShTypes], rfmap[kShTypes], vmap[kShTypes];
  float2 qc[kShTypes], cg[kShTypes], esv[kShTypes];
  int pidx[kShPidx];
  PairFF ppff[kShPairs];
};

// Every thread of the block; the caller synchronises before use.
__device__ void load_tabs(const KP &p, GrandTabs &t, TypeRefs &tr, PairRefs &pr) {
  const bool types = p.ntype + 1 <= kShTypes && p.nttyp + 1 <= kShTypes;
  const bool pairs = types && p.nttyp * p.nttyp <= kShPidx && p.ntc <= kShPairs;
  if (types) {
    for (int i = threadIdx.x; i <= p.ntype; i += blockDim.x) {
      t.nwtype[i] = p.nwtype[i];
      t.qc[i] = p.qcff[i];
      t.cg[i] = p.cgff[i];
      t.rfmap[i] = p.rfpar_map_of_type ? p.rfpar_map_of_type[i] : 0;
      t.vmap[i] = p.phiv_map_of_type ? p.phiv_map_of_type[i] : 0;
    }
    for (int i = threadIdx.x; i <= p.nttyp; i += blockDim.x)
      t.esv[i] = p.esvff ? p.esvff[i] : make_float2(0.f, 0.f);
  }
  if (pairs) {
    for (int i = threadIdx.x; i < p.nttyp * p.nttyp; i += blockDim.x) t.pidx[i] = p.pidx[i];
    const int *src = reinterpret_cast<const int *>(p.ppff);
    int *dst = reinterpret_cast<int *>(t.ppff);
    for (int i = threadIdx.x; i < p.ntc * (int)(sizeof(PairFF) / sizeof(int)); i += blockDim.x)
      dst[i] = src[i];
  }
  tr = types ? TypeRefs{t.nwtype, t.rfmap, t.vmap, t.qc, t.cg, t.esv}
             : TypeRefs{p.nwtype, p.rfpar_map_of_type, p.phiv_map_of_type, p.qcff, p.cgff, p.esvff};
  pr = pairs ? PairRefs{t.pidx, tr.nwtype, t.ppff} : PairRefs{p.pidx, p.nwtype, p.ppff};
}

// rfpar_ifir through the refs
__device__ __forceinline__ size_t rf_ifir(const KP &p, const TypeRefs &tr, int itype) {
  return p.qrfpsin ? 0 : (size_t)tr.rfmap[itype] * ((size_t)p.g3.nclx * p.g3.ncly * p.g3.nclz);
}

// ---- ΔE terms in float-float (ffmath.cuh) -----------------------------------
// GRAND evaluates INTERACT's O(N) terms, the trial-trial terms and their sums
// in float-float; a pair closer than kFFMinD2 falls back to the FP64 law.

constexpr float kFFMinD2 = 0.01f;  // A^2: below, LJ and SRPMF may leave float's range

// Float-float exp and cos stay out of line (one copy each): GRAND's chains
// run once per launch, and inlined copies at every call site stall its
// warps on instruction fetch.  (Routines that read the parameter block stay
// inline: a call would take its address and move it to local memory.)
__device__ __noinline__ f2 exp_ff(f2 a) { return f2_exp(a); }
__device__ __noinline__ f2 cos_ff(f2 a) { return f2_cos(a); }

__device__ __forceinline__ f2 f2_ld(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ float2 f2_st(f2 a) { return make_float2(a.h, a.l); }
__device__ __forceinline__ bool f2_lt(f2 a, f2 b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool f2_le(f2 a, f2 b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); }
__device__ __forceinline__ f2 f2_pow3(f2 v) { return f2_mul(f2_sqr(v), v); }
__device__ __forceinline__ f2 f2_pow6(f2 v) {
  const f2 s = f2_sqr(v);
  return f2_mul(f2_sqr(s), s);
}
// (int) of the value h + l, truncating toward zero as the FP64 code does
__device__ __forceinline__ int f2_trunc(f2 a) {
  int i = (int)a.h;
  if ((float)i == a.h) {
    if (a.h > 0.0f && a.l < 0.0f) --i;
    else if (a.h < 0.0f && a.l > 0.0f) ++i;
  }
  return i;
}
// d - L rint(d / L): the nearest image (the quotient's rounding at an exact
// half box is where the two images are equally near)
__device__ __forceinline__ f2 min_image_ff(f2 d, float2 L, float iL) {
  const float k = rintf(__fmul_rn(d.h, iL));
  return f2_sub(d, f2_mulf(f2_ld(L), k));
}

// efp64 in float-float (polynom.f90:197-230)
__device__ f2 efp_ff(const KP &p, const PairFF &q, f2 x2, int &err) {
  if (f2_lt(x2, f2_ld(q.dm2lo))) {
    const f2 ix2 = f2_rcp(x2);
    return f2_add(f2_mul(f2_ld(q.sc0), f2_pow6(ix2)), f2_ld(q.sc1));
  }
  if (f2_lt(f2_ld(q.dm2hi), x2)) {
    const f2 ix2 = f2_rcp(x2);
    const f2 c = f2_mul(f2_ld(q.sc2), f2_pow3(ix2));
    return (q.flags & kChr) ? f2_add(c, f2_mul(f2_ld(q.fct), f2_sqrt(ix2))) : c;
  }
  const f2 x = f2_sqrt(x2);
  int i = f2_trunc(f2_mul(f2_sub(x, f2_ld(q.dmi)), f2_ld(p.ffc.ires))) + q.nxi;
  if (i < q.nxi || i >= q.nxi + q.npieces) {
    err |= kErrTableIndex;
    i = min(max(i, q.nxi), q.nxi + q.npieces - 1);
  }
  const f2 p1 = f2_ld(p.epff[3 * i]), p2 = f2_ld(p.epff[3 * i + 1]),
           p3 = f2_ld(p.epff[3 * i + 2]);
  return f2_add(p1, f2_mul(x, f2_add(p2, f2_mul(x, p3))));
}

// law_interact64 in float-float: U of a pair at squared distance d2
// (interact.f90's pair terms: Coulomb, LJ, SRPMF, or the tabulated law)
__device__ f2 law_ff(const KP &p, const PairFF &q, f2 d2, int &err) {
  if (q.flags & kEfp) return efp_ff(p, q, d2, err);
  const f2 idist = f2_rsqrt(d2), idist2 = f2_sqr(idist);
  f2 u = f2_f(0.0f);
  if (q.flags & kChr) u = f2_mul(f2_ld(q.fct), idist);
  if (q.flags & kLj) {
    const f2 d6 = f2_pow3(f2_mul(f2_ld(q.sgp2), idist2));
    u = f2_add(u, f2_mul(f2_mul(f2_ld(q.epp4), d6), f2_addf(d6, -1.0f)));
  }
  if ((q.flags & kSrp) && f2_le(d2, f2_ld(p.ffc.rth))) {
    const f2 r = f2_mul(d2, idist);
    const f2 t = f2_sub(f2_ld(q.c1), r);
    f2 es = f2_mul(f2_mul(f2_ld(q.c0), exp_ff(f2_mul(t, f2_ld(q.c2)))),
                   cos_ff(f2_mul(f2_ld(q.c3pi), t)));
    es = f2_add(es, f2_mul(f2_ld(q.c4), f2_pow6(f2_mul(f2_ld(q.c1), idist))));
    const f2 srpx = f2_ld(p.ffc.srpx);
    if (!f2_lt(r, srpx))
      es = f2_sub(f2_mul(es, exp_ff(f2_neg(f2_mul(f2_ld(p.ffc.srpk), f2_sub(r, srpx))))),
                  f2_ld(p.ffc.srpy));
    u = f2_add(u, es);
  }
  return u;
}

// What a GRAND pair term reads of a particle, in float-float: position,
// signed type, RFPAR record (q srfe reff, reff^2).
struct PartFF {
  f2 x, y, z;
  int ti;
  float4 rf;
};

__device__ __forceinline__ PartFF load_partff(const KP &p, int i, bool rf, bool ff) {
  PartFF r;
  r.ti = __ldcg(p.typei + i);
  if (ff) {
    const float4 h = __ldcg(p.pk1 + i), l = __ldcg(p.pk2 + i);
    r.x = {h.x, l.x};
    r.y = {h.y, l.y};
    r.z = {h.z, l.z};
  } else {
    r.x = f2_of(__ldcg(p.x + i));
    r.y = f2_of(__ldcg(p.y + i));
    r.z = f2_of(__ldcg(p.z + i));
  }
  r.rf = rf && i >= p.nsites ? __ldcg(p.gc_rff + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  return r;
}

// The FP64 term of a pair closer than float-float's range (rare)
__device__ double near_pair64(const KP &p, const Trial &tr, uint32_t mask, int i,
                                           int jt2, bool rf, const PartRec &q, int &err) {
  return interact_rec(p, tr, mask, i, jt2, tr.j - 1 >= p.nsites, rf, q, err);
}

// interact_rec in float-float: particle i's ΔE term with trial t.  False
// when the pair is closer than kFFMinD2 (the caller takes the FP64 law).
__device__ __forceinline__ bool pair_ff(const KP &p, const PairRefs &P, const TrialFF &t,
                                        uint32_t mask, int i, const PartFF &q, f2 &u, int &err) {
  u = f2_f(0.0f);
  const bool ion_i = i >= p.nsites;
  const int ti = q.ti;
  if (ion_i && guard_bad(p.st, abs(ti) - p.nold - 1, p.ntype - p.nold, 31)) return true;
  f2 dx = f2_sub(q.x, f2_ld(t.x)), dy = f2_sub(q.y, f2_ld(t.y)), dz = f2_sub(q.z, f2_ld(t.z));
  if (p.periodic) {  // extension mode: nearest image, plain cutoff
    dx = min_image_ff(dx, p.ffc.L[0], p.ffc.iL[0]);
    dy = min_image_ff(dy, p.ffc.L[1], p.ffc.iL[1]);
    dz = min_image_ff(dz, p.ffc.L[2], p.ffc.iL[2]);
  }
  const f2 d2 = f2_add(f2_add(f2_sqr(dx), f2_sqr(dy)), f2_sqr(dz));
  if (p.periodic && !f2_lt(d2, f2_ld(p.ffc.rc2))) return true;
  if (d2.h < kFFMinD2) return false;
  const bool beion = t.j - 1 >= p.nsites;
  if (mask & 1u) {
    int is = -1;
    if (beion && ion_i)  // interact.f90:173-210
      is = P.pidx[(P.nwtype[abs(ti)] - 1) * p.nttyp + t.jt2 - 1];
    else if (beion && !ion_i)  // interact.f90:351-381
      is = P.pidx[(p.typtyp[i] - 1) * p.nttyp + t.jt2 - 1];
    else if (!beion && ion_i)  // interact.f90:383-413
      is = P.pidx[(P.nwtype[abs(ti)] - 1) * p.nttyp + t.jt2 - 1];
    if (is >= 0) u = law_ff(p, P.ppff[is], d2, err);
  }
  if (t.rf && ion_i && q.rf.x != 0.0f) {  // RFPAR cross term
    const f2 c = {q.rf.x, q.rf.y}, rr = {q.rf.z, q.rf.w};
    u = f2_add(u, f2_mul(f2_mul(f2_ld(t.a), c), f2_rsqrt(f2_add(f2_mul(f2_ld(t.b), rr), d2))));
  }
  return true;
}

// ---- single-particle terms in float-float ----------------------------------
__device__ __forceinline__ f2 f2_abs(f2 a) { return a.h < 0.0f ? f2_neg(a) : a; }

__device__ __forceinline__ bool in_grid_ff(const GridFF &g, f2 x, f2 y, f2 z) {
  return f2_le(x, f2_ld(g.ub[0])) && f2_le(f2_ld(g.lb[0]), x) && f2_le(y, f2_ld(g.ub[1])) &&
         f2_le(f2_ld(g.lb[1]), y) && f2_le(z, f2_ld(g.ub[2])) && f2_le(f2_ld(g.lb[2]), z);
}

// cell_of: the cell of grid coordinate xi (truncated), clamped below the
// last node
__device__ __forceinline__ int cell_ff(const GridFF &g, f2 xi, int a) {
  const int i = f2_trunc(f2_mul(xi, f2_ld(g.idcel)));
  return i == g.ncl[a] - 1 ? g.ncl[a] - 2 : i;
}

// spln_cell: the nearest node (half away from zero), clamped to the interior
__device__ __forceinline__ int spln_node_ff(const GridFF &g, f2 xi, int a) {
  const f2 u = f2_mul(xi, f2_ld(g.idcel));
  int n = (int)floorf(u.h);
  f2 r = f2_addf(u, -(float)n);  // u - n, exact
  if (r.h < 0.0f) {
    --n;
    r = f2_addf(r, 1.0f);
  }
  const f2 half = f2_f(0.5f);
  if (f2_lt(half, r) || (r.h == 0.5f && r.l == 0.0f && n >= 0)) ++n;
  if (n == 0) n = 1;
  if (n == g.ncl[a] - 1) n = g.ncl[a] - 2;
  return n;
}

// 1 - |xi - node dcel| / dcel: the trilinear weight of a node along one axis
__device__ __forceinline__ f2 tri_w(const GridFF &g, f2 xi, int node) {
  const f2 d = f2_abs(f2_sub(xi, f2_mulf(f2_ld(g.dcel), (float)node)));
  return f2_sub(f2_f(1.0f), f2_mul(d, f2_ld(g.idcel)));
}

// quadratic B-spline m3 (m3.f90)
__device__ __forceinline__ f2 m3_ff(f2 x) {
  const f2 zero = f2_f(0.0f);
  const bool in02 = f2_le(zero, x) && f2_le(x, f2_f(2.0f));
  const bool in13 = f2_le(f2_f(1.0f), x) && f2_le(x, f2_f(3.0f));
  const f2 m2m = in02 ? f2_sub(f2_f(1.0f), f2_abs(f2_addf(x, -1.0f))) : zero;
  const f2 m2 = in13 ? f2_sub(f2_f(1.0f), f2_abs(f2_addf(x, -2.0f))) : zero;
  if (!(f2_le(zero, x) && f2_le(x, f2_f(3.0f)))) return zero;
  return f2_add(f2_mul(f2_mulf(x, 0.5f), m2m), f2_mul(f2_mulf(f2_sub(f2_f(3.0f), x), 0.5f), m2));
}

__device__ __forceinline__ f2 shfl_xor_ff(f2 v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}
__device__ __forceinline__ f2 seg8_ff(f2 v) {
  v = f2_add(v, shfl_xor_ff(v, 4));
  v = f2_add(v, shfl_xor_ff(v, 2));
  return f2_add(v, shfl_xor_ff(v, 1));
}
__device__ __forceinline__ f2 wsum_ff(f2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = f2_add(v, shfl_xor_ff(v, o));
  return v;
}

// rfpar_gather (rfpar.f90:94-150, no gradients, the same early exit) in
// float-float: (srfe, reff) of an ion of the map ifir at (x, y, z); (0, 0)
// off the map, as rf_single.
__device__ void rf_gather_ff(const KP &p, f2 x, f2 y, f2 z, size_t ifir, f2 &srfe, f2 &reff) {
  const GridFF &g = p.ffc.g[2];
  srfe = reff = f2_f(0.0f);
  if (!in_grid_ff(g, x, y, z)) return;
  const f2 xi = f2_add(x, f2_ld(g.o[0])), yi = f2_add(y, f2_ld(g.o[1])),
           zi = f2_add(z, f2_ld(g.o[2]));
  const int ix = cell_ff(g, xi, 0), iy = cell_ff(g, yi, 1), iz = cell_ff(g, zi, 2);
  const size_t ncyz = (size_t)g.ncl[1] * g.ncl[2];
  const f2 sq = f2_ld(p.ffc.sqrfac);
  float gs[8], gr[8];  // the eight nodes' values, loaded together
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const size_t node = ifir + (size_t)(ix + (n >> 2)) * ncyz +
                        (size_t)(iy + ((n >> 1) & 1)) * g.ncl[2] + iz + (n & 1);
    gs[n] = __ldg(p.gsrfen + node);
    gr[n] = __ldg(p.greff + node);
  }
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const f2 ai = tri_w(g, xi, ix + a);
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const f2 ab = f2_mul(ai, tri_w(g, yi, iy + b));
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int n = 4 * a + 2 * b + c;
        if (gs[n] == 0.0f) break;  // the reference's exit of the innermost loop
        const f2 fi = f2_mul(ab, tri_w(g, zi, iz + c));
        srfe = f2_add(srfe, f2_mulf(fi, gs[n]));
        reff = f2_add(reff, f2_mul(fi, f2_mulf(sq, gr[n])));
      }
    }
  }
}

// RFPAR record (q srfe reff, reff^2) of an ion of type |ti|
__device__ __forceinline__ float4 rf_record_ff(const TypeRefs &tr, f2 srfe, f2 reff, int ti) {
  const f2 c = f2_mul(f2_mul(f2_ld(tr.cg[abs(ti)]), srfe), reff), d = f2_sqr(reff);
  return make_float4(c.h, c.l, d.h, d.l);
}

// trial_single_warp in float-float for an ion trial at (x, y, z) (one full
// warp, the same lane layout: lanes 8g + corner the trilinear nodes of the
// static field, the repulsion map, gsrfen and greff; lanes 0..26 the
// B-spline nodes); the membrane term stays FP64 (lane 0).  Lane 0 fills
// tr.e_single, srfe, reff, rf_in and returns srfe, reff in float-float.
__device__ void trial_single_ff(const KP &p, const TypeRefs &T, Trial &tr, f2 x, f2 y, f2 z,
                                uint32_t mask, int qalert, int *nalert, f2 &srfe_o, f2 &reff_o,
                                f2 &e_o) {
  const int lane = threadIdx.x & 31;
  const FFC &c = p.ffc;
  const int j0 = tr.j - 1, it = tr.itype;
  const int jt2 = T.nwtype[it];
  const int g = lane >> 3, cn = lane & 7;
  const int ca = (cn >> 2) & 1, cb = (cn >> 1) & 1, cc = cn & 1;
  const bool do_phix = (mask & 4u) && p.qphix && in_grid_ff(c.g[0], x, y, z);
  const GridFF &g2 = c.g[1];
  const bool do_phiv = (mask & 8u) && p.qphiv && f2_le(x, f2_ld(g2.ub[0])) &&
                       f2_le(f2_ld(g2.lb[0]), x) && f2_le(y, f2_ld(g2.ub[1])) &&
                       f2_le(f2_ld(g2.lb[1]), y) && f2_le(z, f2_ld(c.vzmax)) &&
                       f2_le(f2_ld(c.vzmin), z);
  const bool do_rf = (mask & 16u) && p.qrfpar && in_grid_ff(c.g[2], x, y, z);
  // repulsion map and scale (phiv_select for an ion slot)
  size_t vifir = 0;
  if (p.qnmcden && j0 >= p.nsites + p.nfix)
    vifir = (size_t)T.vmap[it] * ((size_t)p.g2.nclx * p.g2.ncly * p.g2.nclz);
  const f2 esv = do_phiv ? f2_ld(T.esv[jt2]) : f2_f(0.0f);
  const f2 qc = f2_ld(T.qc[it]);
  const size_t rfifir = do_rf ? rf_ifir(p, T, it) : 0;
  f2 v = f2_f(0.0f), w = f2_f(0.0f);
  float psum = 0.0f, gs_own = 0.0f;
  bool active = false;
  if ((g == 0 && do_phix) || (g == 1 && do_phiv && p.qtrln) || (g >= 2 && do_rf)) {
    const GridFF &gg = c.g[g == 0 ? 0 : (g == 1 ? 1 : 2)];
    const f2 xi = f2_add(x, f2_ld(gg.o[0])), yi = f2_add(y, f2_ld(gg.o[1])),
             zi = f2_add(z, f2_ld(gg.o[2]));
    const int ix = cell_ff(gg, xi, 0), iy = cell_ff(gg, yi, 1), iz = cell_ff(gg, zi, 2);
    w = f2_mul(f2_mul(tri_w(gg, xi, ix + ca), tri_w(gg, yi, iy + cb)), tri_w(gg, zi, iz + cc));
    const size_t node = (size_t)(ix + ca) * gg.ncl[1] * gg.ncl[2] +
                        (size_t)(iy + cb) * gg.ncl[2] + iz + cc;
    if (g == 0) {
      v = f2_mulf(qc, __ldg(p.phix + node));
    } else if (g == 1) {
      psum = (float)__ldg(p.phiv + vifir + node);
      v = f2_mulf(esv, psum);
    } else {
      const size_t n3 = rfifir + node;
      gs_own = __ldg(p.gsrfen + n3);
      v = g == 2 ? f2_f(gs_own) : f2_mulf(f2_ld(c.sqrfac), __ldg(p.greff + n3));
    }
    active = true;
  }
  const float gs_c0 = __shfl_sync(0xffffffffu, gs_own, lane & ~1);
  if (g >= 2 && active && !(gs_c0 != 0.0f && (cc == 0 || gs_own != 0.0f))) active = false;
  f2 le = active ? f2_mul(w, v) : f2_f(0.0f);
  le = seg8_ff(le);
  psum += __shfl_xor_sync(0xffffffffu, psum, 4);  // at most 8 small integers: exact
  psum += __shfl_xor_sync(0xffffffffu, psum, 2);
  psum += __shfl_xor_sync(0xffffffffu, psum, 1);
  f2 be = f2_f(0.0f);
  float bsum = 0.0f;
  if (do_phiv && !p.qtrln) {  // warp-uniform
    f2 e1 = f2_f(0.0f);
    float s1 = 0.0f;
    if (lane < 27) {
      const f2 xi = f2_add(x, f2_ld(g2.o[0])), yi = f2_add(y, f2_ld(g2.o[1])),
               zi = f2_add(z, f2_ld(g2.o[2]));
      const int ix = spln_node_ff(g2, xi, 0), iy = spln_node_ff(g2, yi, 1),
                iz = spln_node_ff(g2, zi, 2);
      const int k = ix - 1 + lane / 9, l = iy - 1 + (lane / 3) % 3, m = iz - 1 + lane % 3;
      const f2 dc = f2_ld(g2.dcel), id = f2_ld(g2.idcel);
      auto arg = [&](f2 q, int n) {
        return f2_sub(f2_f(1.5f), f2_mul(f2_sub(q, f2_mulf(dc, (float)n)), id));
      };
      const f2 fi = f2_mul(f2_mul(m3_ff(arg(xi, k)), m3_ff(arg(yi, l))), m3_ff(arg(zi, m)));
      if (fi.h != 0.0f) {
        const float phis = (float)__ldg(p.phiv + vifir + (size_t)k * g2.ncl[1] * g2.ncl[2] +
                                        (size_t)l * g2.ncl[2] + m);
        s1 = phis;
        e1 = f2_mulf(f2_mul(fi, esv), phis);
      }
    }
    be = wsum_ff(e1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s1 += __shfl_xor_sync(0xffffffffu, s1, o);  // exact
    bsum = s1;
  }
  const f2 e_v = {__shfl_sync(0xffffffffu, le.h, 8), __shfl_sync(0xffffffffu, le.l, 8)};
  const float s_v = __shfl_sync(0xffffffffu, psum, 8);
  const f2 sj = {__shfl_sync(0xffffffffu, le.h, 16), __shfl_sync(0xffffffffu, le.l, 16)};
  const f2 rj = {__shfl_sync(0xffffffffu, le.h, 24), __shfl_sync(0xffffffffu, le.l, 24)};
  if (lane == 0) {
    f2 e = f2_f(0.0f);
    if ((mask & 2u) && p.qmemb) {  // FP64
      double em = 0.0, f[3];
      if (membrane_one(p, jt2, p.cg[it], tr.x, tr.y, tr.z, false, true, em, f) && qalert) {
        if (nalert)
          ++*nalert;
        else
          atomicAdd(&p.warn[jt2], 1);
      }
      e = f2_of(em);
    }
    if (do_rf)
      e = f2_add(e, f2_mulf(f2_mul(f2_mul(qc, f2_ld(T.cg[it])), f2_sqr(sj)), 0.5f));
    if (do_phix) e = f2_add(e, le);
    if (do_phiv) {
      f2 ev = p.qtrln ? e_v : be;
      const float ps = p.qtrln ? s_v : bsum;
      if (f2_le(f2_ld(p.qtrln ? c.thold8 : c.thold27), f2_f(ps))) {
        ev = f2_f(1.0e10f);  // exact in float
        if (qalert) {
          if (nalert)
            ++*nalert;
          else
            atomicAdd(&p.warn[jt2], 1);
        }
      }
      e = f2_add(e, ev);
    }
    tr.e_single = f2_dbl(e);
    e_o = e;
    srfe_o = do_rf ? sj : f2_f(0.0f);
    reff_o = do_rf ? rj : f2_f(0.0f);
    tr.srfe = f2_dbl(srfe_o);
    tr.reff = f2_dbl(reff_o);
    tr.rf_in = do_rf ? 1 : 0;
  }
}

// A trial as the pair terms read it (block 0, once per trial), from its
// float-float position and RFPAR gathers.
__device__ TrialFF trial_ff(const KP &p, const TypeRefs &T, const Trial &t, uint32_t mask, f2 x,
                            f2 y, f2 z, f2 srfe, f2 reff) {
  TrialFF f{};
  f.valid = t.valid;
  f.j = t.j;
  f.jt2 = trial_type2(p, t);
  f.rf = t.valid && t.rf_in && (mask & 16u);
  f.x = f2_st(x);
  f.y = f2_st(y);
  f.z = f2_st(z);
  if (f.rf) {
    f.a = f2_st(f2_mul(f2_mul(f2_ld(T.qc[t.itype]), srfe), reff));
    f.b = f2_st(f2_sqr(reff));
  }
  return f;
}

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
  f2 fx[kSpec], fy[kSpec], fz[kSpec];  // the trials' positions in float-float
  f2 fsr[kSpec], fre[kSpec];            // and their RFPAR gathers (srfe, reff)
  TrialFF tf[kSpec];        // the trials as the pair terms read them
  // each trial's particle as an ion record holds it: position (that of the
  // float-float record in FP32 mode), signed type, RFPAR record, and the
  // RFPAR gathers behind it
  PartFF pff[kSpec];
  f2 psr[kSpec], pre_[kSpec];
  int ti[kSpec];
  f2 es[kSpec];             // the trials' single-particle terms
  f2 tt[kSpec][kSpec];      // tt[k][a], k < a: trial a's pair term with k's particle
  int terr[kSpec][kSpec];
  f2 base[kSpec];           // the round's sums, totalled over the blocks
  int aerr[kSpec];
  f2 uacc[kSpec];           // the acceptance draws (exact in float-float)
  int dti[kSpec];           // a deletion target's signed type
  // settling in waves: per attempt its outcome in the current state, its ΔE
  // and error flags; the moves accepted so far in the round
  int wst[kSpec], werr[kSpec];
  f2 wde[kSpec];
  int cur, stop, nacc, acck[kSpec], accs[kSpec];
  unsigned long long touched;  // bit b: an accepted deletion touched buffer b + 1
  f2 avf[kMaxBuffers + 1], muf[kMaxBuffers + 1], kbbf[kMaxBuffers + 1];
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
// drawn from (find.f90).  None depends on the state.  S: the buffer
// parameters (nbuf, and 1-based avnum, ibfftyp, lzmin, lzmax, rmin, rmax).
template <class S>
__device__ void propose_draws(const KP &p, uint64_t seed, uint64_t cycle, uint32_t attempt,
                              const S &g, Trial &t, double &u_rank) {
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
__device__ void build_round(const KP &p, const TypeRefs &T, uint32_t mask, uint64_t seed,
                            uint64_t cycle, int a0, int na, GrandState &g) {
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
    {  // the same draw in float-float: word * 2^-32 split at bit 8, exact
      const uint32_t w = gcmc_word(seed, cycle, (uint32_t)(a0 + t), (uint32_t)tr.draw);
      float h, l;
      two_sum((float)(w & 0xFFFFFF00u) * 0x1p-32f, (float)(w & 0xFFu) * 0x1p-32f, h, l);
      g.uacc[t] = {h, l};
    }
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
  if (t < na) {  // positions in float-float: a deletion's from its records
    const Trial &tr = g.tr[t];
    g.dti[t] = tr.valid && !tr.insert ? __ldcg(p.typei + tr.j - 1) : 0;
    if (tr.valid && !tr.insert && g.ff) {
      const int k = tr.j - 1;
      const float4 h = __ldcg(p.pk1 + k), l = __ldcg(p.pk2 + k);
      g.fx[t] = {h.x, l.x};
      g.fy[t] = {h.y, l.y};
      g.fz[t] = {h.z, l.z};
    } else {
      g.fx[t] = f2_of(tr.x);
      g.fy[t] = f2_of(tr.y);
      g.fz[t] = f2_of(tr.z);
    }
    g.fsr[t] = g.fre[t] = f2_f(0.0f);
  }
  __syncthreads();
  for (int k = t >> 5; k < na; k += kGrandWarps) {
    Trial tr = g.tr[k];
    if (tr.valid) {
      f2 sr, re, es;
      trial_single_ff(p, T, tr, g.fx[k], g.fy[k], g.fz[k], mask, tr.insert ? 0 : 1, &g.nalert[k],
                      sr, re, es);
      if ((t & 31) == 0) {
        g.es[k] = es;
        g.tr[k].e_single = tr.e_single;
        g.tr[k].srfe = tr.srfe;
        g.tr[k].reff = tr.reff;
        g.tr[k].rf_in = tr.rf_in;
        g.fsr[k] = sr;
        g.fre[k] = re;
      }
    }
  }
  __syncthreads();
  if (t < na)
    g.tf[t] = trial_ff(p, T, g.tr[t], mask, g.fx[t], g.fy[t], g.fz[t], g.fsr[t], g.fre[t]);
  __syncthreads();
}

// A coordinate as its float-float record stores it (hi = fl(x), lo =
// fl(x - hi)), read back as hi + lo.
__device__ __forceinline__ double ff_rounded(double x) {
  const float h = (float)x;
  return (double)h + (double)(float)(x - (double)h);
}

// Each trial's particle as an ion record holds it (block 0, a thread per
// trial): an insertion's what its acceptance writes (the point as its
// record holds it, the signed type, the RFPAR record at that point), a
// deletion's its target's record.  The RFPAR gathers at that point are the
// trial's own (trial_single_ff, the same map nodes and early exit).
__device__ void trial_ions(const KP &p, const TypeRefs &T, uint32_t mask, int na,
                           GrandState &g) {
  const int t = threadIdx.x;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  if (t < na) {
    const Trial &tr = g.tr[t];
    const int ti = !tr.valid ? 0 : (tr.insert ? (tr.z < p.cz ? -tr.itype : tr.itype) : g.dti[t]);
    g.ti[t] = ti;
    g.psr[t] = g.fsr[t];
    g.pre_[t] = g.fre[t];
    PartFF &q = g.pff[t];
    q.x = g.fx[t];
    q.y = g.fy[t];
    q.z = g.fz[t];
    q.ti = ti;
    q.rf = tr.valid && rf_on ? rf_record_ff(T, g.fsr[t], g.fre[t], ti)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Trial-trial pair terms (block 0, a thread per pair k < a): trial a's
// INTERACT term with trial k's particle as an ion record holds it.
__device__ void trial_pairs(const KP &p, const PairRefs &P, uint32_t mask, int na,
                            GrandState &g) {
  for (int idx = threadIdx.x; idx < na * na; idx += blockDim.x) {
    const int k = idx / na, a = idx - k * na;
    if (k >= a) continue;
    const Trial &ta = g.tr[a], &tk = g.tr[k];
    f2 v = f2_f(0.0f);
    int err = 0;
    // two deletions of one ion are never both settled (the first touches
    // the buffer of the second)
    if (ta.valid && tk.valid && (ta.insert || tk.insert || ta.j != tk.j)) {
      const TrialFF &fa = g.tf[a];
      if (fa.jt2 > 0) {
        if (!pair_ff(p, P, fa, mask, p.nsites, g.pff[k], v, err)) {  // closer than float-float's range: the FP64 law
          PartRec q;
          q.x = f2_dbl(g.pff[k].x);
          q.y = f2_dbl(g.pff[k].y);
          q.z = f2_dbl(g.pff[k].z);
          q.rf = make_double2(f2_dbl(g.psr[k]), f2_dbl(g.pre_[k]));
          q.ti = g.ti[k];
          v = f2_of(near_pair64(p, ta, mask, p.nsites, fa.jt2, fa.rf != 0, q, err));
        }
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
  const float2 *ipf = reinterpret_cast<const float2 *>(p.ipart);
  for (int a = threadIdx.x >> 5; a < na; a += kGrandWarps) {
    f2 v = f2_f(0.0f);
    int e = 0;
    for (int b = 1 + lane; b < nblk; b += 32) {
      v = f2_add(v, f2_ld(__ldcg(ipf + (size_t)b * kSpec + a)));
      e |= __ldcg(p.ierr + (size_t)b * kSpec + a);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      v = f2_add(v, {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)});
    e = __reduce_or_sync(0xffffffffu, e);
    if (lane == 0) {
      g.base[a] = v;
      g.aerr[a] = e;
    }
  }
}

// Im-Roux acceptance probability of trial tr with total ΔE de in the
// current state (grand.f90:88-116).  S: the counts (0-based nat, ntotat)
// and the 1-based buffer parameters (avnum, mu, kbb, qbias).
template <class S>
__device__ double accept_rate(const KP &p, const S &g, const Trial &tr, double de,
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

// accept_rate's decision in float-float: 1 accept, 0 reject, -1 when the
// Boltzmann factor's exponent leaves float's range (decide in FP64).  The
// draw u is exact; the rate agrees with the FP64 one to ~2^-46, so the two
// decisions differ only for draws that close to the rate.
__device__ int accept_ff(const KP &p, const GrandState &g, const Trial &tr, f2 de, f2 u,
                         uint64_t cycle) {
  const int ib = tr.ib, b = ib - 1;
  const int nat = g.nat[b];
  const f2 x = f2_neg(f2_mul(f2_sub(de, g.muf[ib]), f2_ld(p.ffc.ikbt)));
  if (!(fabsf(x.h) <= 80.0f)) return -1;  // also NaN
  const f2 boltz = exp_ff(x);
  f2 a = g.avf[ib];
  if (g.qbias[ib])
    a = f2_add(a, f2_mul(g.kbbf[ib], f2_addf(a, -(float)(g.ntotat[b] / (long long)cycle))));
  f2 rate;
  if (tr.insert) {
    rate = f2_div(f2_mul(a, boltz), f2_f((float)(nat + 1)));
    rate = f2_div(rate, f2_addf(rate, 1.0f));
  } else {
    rate = f2_div(f2_mul(a, boltz), f2_f((float)nat));
    rate = f2_rcp(f2_addf(rate, 1.0f));
  }
  return f2_le(u, rate) ? 1 : 0;
}

__device__ __forceinline__ bool accepts(const KP &p, const GrandState &g, const Trial &tr, f2 de,
                                        int a, uint64_t cycle) {
  const int r = accept_ff(p, g, tr, de, g.uacc[a], cycle);
  return r >= 0 ? r != 0 : g.u_acc[a] <= accept_rate(p, g, tr, f2_dbl(de), cycle);
}

// Outcomes of an attempt in the current state.
enum : int { kNoop = 0, kReject = 1, kAccept = 2, kStop = 3 };

// One attempt in the current state (block 0, the attempt's thread): kStop
// when its deletion trial may no longer name its target (a new round
// proposes it), kNoop when there is nothing to do, else its acceptance,
// with ΔE -- the round's sum plus the trial-trial terms of the moves
// accepted so far -- and the error flags of the terms it used.
__device__ int evaluate(const KP &p, uint64_t cycle, int a, GrandState &g, f2 &de, int &err) {
  const Trial &tr = g.tr[a];
  de = f2_f(0.0f);
  err = 0;
  bool valid = tr.valid;
  if (g.nacc > 0 && !tr.insert) {  // the deletion trial in the current state
    const int ib = tr.ib;
    const int natb = ib <= g.nbuf ? g.nat[ib - 1] : 0;
    const int ip = (int)((double)natb * g.u_rank[a]) + 1;
    if (!(ib <= g.nbuf && ip <= natb))
      valid = false;  // no ion left to delete
    else if (g.ip0[a] == 0 || ip != g.ip0[a] || ((g.touched >> (ib - 1)) & 1ull))
      return kStop;
  }
  if (!valid || guard_bad(p.st, tr.ib - 1, p.nbuffer, 21)) return kNoop;
  err = g.aerr[a];
  de = f2_add(g.es[a], g.base[a]);
  for (int m = 0; m < g.nacc; ++m) {
    const f2 t = g.tt[g.acck[m]][a];
    de = f2_add(de, g.accs[m] > 0 ? t : f2_neg(t));
    err |= g.terr[g.acck[m]][a];
  }
  return accepts(p, g, tr, de, a, cycle) ? kAccept : kReject;
}

// The insertion or deletion of accepted attempt a (grand.f90:63-110; block
// 0, thread 0).  False when nothing changed (capacity or a guard).
__device__ bool apply_move(const KP &p, bool rf_on, int a, GrandState &g) {
  const Trial &tr = g.tr[a];
  const f2 de = g.wde[a];
  const int ib = tr.ib, b = ib - 1;
  const int ntot = g.ntot, nat = g.nat[b];
  if (tr.insert) {
    if (ntot + 1 > p.cap) {
      atomicOr(&p.st->err, kErrCapacity);
      return false;
    }
    if (guard_bad(p.st, ntot, p.cap, 22)) return false;
    g.dener_sum += f2_dbl(de);
    g.nat[b] = nat + 1;
    if (g.ff) {  // the records as k_pack forms them (a mobile ion)
      const f2 x = g.fx[a], y = g.fy[a], z = g.fz[a];
      const int code = (p.nwtype[tr.itype] - 1) | (1 << 16);
      p.pk1[ntot] = make_float4(x.h, y.h, z.h, __int_as_float(code));
      p.pk2[ntot] = make_float4(x.l, y.l, z.l, 0.0f);
      p.pk3[ntot] = make_float4(0.0f, (float)p.cg[tr.itype], __int_as_float(1 << 1), 0.0f);
    } else {
      p.x[ntot] = tr.x;
      p.y[ntot] = tr.y;
      p.z[ntot] = tr.z;
    }
    p.typei[ntot] = g.ti[a];
    p.ibuffer[ntot] = ib;
    if (rf_on) p.gc_rff[ntot] = g.pff[a].rf;
    g.ntot = ntot + 1;
    g.ninsert[b] += 1;
    g.chg[g.nchg++] = ntot;
    g.pdel[a] = 1;
  } else {
    if (guard_bad(p.st, tr.j - 1, ntot, 23) || guard_bad(p.st, ntot - 1, p.cap, 24)) return false;
    const int iat = tr.j - 1, last = ntot - 1;
    // every read of the last ion first, then the writes into the freed slot:
    // the reads then overlap instead of each waiting behind a write
    const int bz = __ldcg(p.ibuffer + last);  // the ion the freed slot receives
    const int tz = __ldcg(p.typei + last);
    float4 r1 = make_float4(0.f, 0.f, 0.f, 0.f), r2 = r1, r3 = r1, rr = r1;
    double dx = 0.0, dy = 0.0, dz = 0.0;
    if (g.ff) {
      r1 = __ldcg(p.pk1 + last);
      r2 = __ldcg(p.pk2 + last);
      r3 = __ldcg(p.pk3 + last);
    } else {
      dx = __ldcg(p.x + last);
      dy = __ldcg(p.y + last);
      dz = __ldcg(p.z + last);
    }
    if (rf_on) rr = __ldcg(p.gc_rff + last);
    g.dener_sum -= f2_dbl(de);
    g.nremove[b] += 1;
    if (g.ff) {
      p.pk1[iat] = r1;
      p.pk2[iat] = r2;
      p.pk3[iat] = r3;
    } else {
      p.x[iat] = dx;
      p.y[iat] = dy;
      p.z[iat] = dz;
    }
    p.typei[iat] = tz;
    p.ibuffer[iat] = bz;
    if (rf_on) p.gc_rff[iat] = rr;
    g.nat[b] = nat - 1;
    g.ntot = ntot - 1;
    g.chg[g.nchg++] = iat;
    g.pdel[a] = -1;
    g.touched |= 1ull << b;
    if (bz >= 1 && bz <= kMaxBuffers) g.touched |= 1ull << (bz - 1);
  }
  g.pbuf[a] = b;
  g.acck[g.nacc] = a;
  g.accs[g.nacc++] = tr.insert ? 1 : -1;
  return true;
}

// The round's attempts in order (block 0, every thread), in waves: each
// wave evaluates every attempt not yet settled, in parallel, in the current
// state; thread 0 then settles them in order up to the first move made
// (the rest are evaluated again in the new state) or the first trial that
// no longer holds (the round ends there).  A wave per accepted move, plus
// one.  g.done: the attempts settled; g.chg: the slots rewritten.
__device__ void settle(const KP &p, uint32_t mask, uint64_t cycle, int na, GrandState &g) {
  const int t = threadIdx.x;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  if (t == 0) {
    g.cur = 0;
    g.stop = 0;
    g.nacc = 0;
    g.touched = 0;
    g.nchg = 0;
  }
  __syncthreads();
  for (;;) {
    const int a0 = g.cur;
    if (a0 >= na || g.stop) break;
    if (t >= a0 && t < na) g.wst[t] = evaluate(p, cycle, t, g, g.wde[t], g.werr[t]);
    __syncthreads();
    if (t == 0) {
      int k = a0;
      while (k < na) {
        const int st = g.wst[k];
        if (st == kStop) {
          g.stop = 1;
          break;
        }
        const Trial &tr = g.tr[k];
        g.pbuf[k] = -1;
        g.pdel[k] = 0;
        if (g.werr[k]) atomicOr(&p.st->err, g.werr[k]);
        if (st != kNoop && !tr.insert && g.nalert[k] > 0)
          atomicAdd(&p.warn[p.nwtype[tr.itype]], g.nalert[k]);
        const bool moved = st == kAccept && apply_move(p, rf_on, k, g);
        ++k;
        if (moved) break;
      }
      g.cur = k;
    }
    __syncthreads();
  }
  if (t == 0) g.done = g.cur;
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
  __shared__ GrandTabs tabs;
  __shared__ float2 red[kGrandWarps * kSpec];
  __shared__ int ered[kGrandWarps * kSpec];
  __shared__ int flag;
  DevState *st = p.st;
  const bool rf_on = (mask & 16u) && p.qrfpar;
  const int ntot0 = st->ntot;
  bool ok = true;
  if (blockIdx.x == 0 && ntot0 > 0 && ntot0 <= p.cap) {
    // into L2 while the tables, the state and the draws are loaded and
    // formed: the buffer tags the deletion-target scan reads (a line of 32
    // a thread), and the last ion's records, which a deletion moves into
    // the freed slot
    const int t = threadIdx.x, last = ntot0 - 1;
    for (int s = p.nsites + p.nfix + 32 * t; s < ntot0; s += 32 * (int)blockDim.x)
      prefetch_l2(p.ibuffer + s);
    if (t == 0) prefetch_l2(p.ibuffer + last);
    if (t == 1) prefetch_l2(p.typei + last);
    if (t == 2) prefetch_l2(ffpos ? (const void *)(p.pk1 + last) : (const void *)(p.x + last));
    if (t == 3) prefetch_l2(ffpos ? (const void *)(p.pk2 + last) : (const void *)(p.y + last));
    if (t == 4) prefetch_l2(ffpos ? (const void *)(p.pk3 + last) : (const void *)(p.z + last));
    if (t == 5 && (mask & 16u) && p.qrfpar) prefetch_l2(p.gc_rff + last);
  }
  TypeRefs T;
  PairRefs P;
  load_tabs(p, tabs, T, P);
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
      g.avf[ib] = f2_ld(p.bufff[3 * ib]);
      g.muf[ib] = f2_ld(p.bufff[3 * ib + 1]);
      g.kbbf[ib] = f2_ld(p.bufff[3 * ib + 2]);
    }
    if (threadIdx.x == 0) {
      g.ntot = ntot0;
      g.dener_sum = 0.0;  // the call's sum
      g.ff = ffpos;
      g.nbuf = nb;
      g.nchg = 0;
      g.nacc = 0;  // evaluate's view before the first settle
      g.touched = 0;
    }
    __syncthreads();
    int a0 = 0;
    for (unsigned r = 1; ok; ++r) {
      const int na = min(ngcmc - a0, kSpec);
      if (na > 0) build_round(p, T, mask, seed, cycle, a0, na, g);
      if (threadIdx.x == kGrandThreads - 32) {  // publish the round (warp 0 goes on)
        GrandRound *hd = p.ground;
        hd->a0 = a0;
        hd->na = na;
        hd->ntot = g.ntot;
        hd->nchg = g.nchg;
        for (int c = 0; c < g.nchg; ++c) hd->chg[c] = g.chg[c];
        for (int k = 0; k < na; ++k) {
          p.trial[k] = g.tr[k];
          p.tff[k] = g.tf[k];
        }
        release_add(&st->bar_gen, 1u);  // orders this thread's stores before it
      }
      if (na <= 0) break;
      trial_ions(p, T, mask, na, g);
      for (int b = threadIdx.x; b < nb; b += blockDim.x) g.nat0[b] = g.nat[b];
      __syncthreads();
      trial_pairs(p, P, mask, na, g);
      if (!(ok = block_wait(&st->bar_count, (unsigned)(gridDim.x - 1) * r, st, &flag))) break;
      round_sums(p, na, g);
      __syncthreads();
      settle(p, mask, cycle, na, g);
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
    launch_exit(st);
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
  float4 rf0 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (rf_on && la == 0)
    for (int i = i0; i < ntot0; i += stride)
      if (i >= p.nsites) {
        const PartFF q = load_partff(p, i, false, ffpos);
        f2 sr, re;
        rf_gather_ff(p, q.x, q.y, q.z, rf_ifir(p, T, abs(q.ti)), sr, re);
        const float4 c = rf_record_ff(T, sr, re, q.ti);
        p.gc_rff[i] = c;
        if (i == i0) rf0 = c;
      }
  PartFF pre{};
  if (i0 < ntot0) pre = load_partff(p, i0, false, ffpos);
  const int src = lane & ~(ap - 1);
  pre.rf = make_float4(__shfl_sync(0xffffffffu, rf0.x, src), __shfl_sync(0xffffffffu, rf0.y, src),
                       __shfl_sync(0xffffffffu, rf0.z, src), __shfl_sync(0xffffffffu, rf0.w, src));
  for (unsigned r = 1; ok; ++r) {
    if (!(ok = block_wait(&st->bar_gen, r, st, &flag))) break;
    // the round header and the lane's trial, loaded together (a trial slot
    // past the round's attempts holds stale data and is not used)
    const GrandRound *hd = p.ground;
    const int na = __ldcg(&hd->na), ntot = __ldcg(&hd->ntot), nchg = __ldcg(&hd->nchg);
    TrialFF tf;
    {
      const uint2 *src2 = reinterpret_cast<const uint2 *>(p.tff + la);
      uint2 *dst2 = reinterpret_cast<uint2 *>(&tf);
#pragma unroll
      for (int k = 0; k < (int)(sizeof(TrialFF) / sizeof(uint2)); ++k) dst2[k] = __ldcg(src2 + k);
    }
    if (na <= 0) break;
    if (la >= na) tf.valid = 0;
    for (int c = 0; c < nchg; ++c)  // the previous round rewrote this slot
      if (__ldcg(&hd->chg[c]) == i0 && i0 < ntot) pre = load_partff(p, i0, rf_on, ffpos);
    f2 u = f2_f(0.0f);
    int err = 0;
    if (tf.valid && tf.jt2 > 0)
      for (int i = i0; i < ntot; i += stride)
        if (i != tf.j - 1) {
          f2 v;
          if (!pair_ff(p, P, tf, mask, i, i == i0 ? pre : load_partff(p, i, rf_on, ffpos), v,
                       err)) {
            // closer than float-float's range: the FP64 law (RFPAR gathered in FP64)
            const Trial tr = load_trial_cg(p.trial + la);
            PartRec q = load_part(p, i, false, ffpos);
            if (rf_on && i >= p.nsites) q.rf = rf_single(p, q.x, q.y, q.z, abs(q.ti));
            v = f2_of(near_pair64(p, tr, mask, i, tf.jt2, tf.rf != 0, q, err));
          }
          u = f2_add(u, v);
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      if (o >= ap) {  // lanes of one attempt
        u = f2_add(u, {__shfl_xor_sync(0xffffffffu, u.h, o), __shfl_xor_sync(0xffffffffu, u.l, o)});
        err |= __shfl_xor_sync(0xffffffffu, err, o);
      }
    if (lane < ap) {
      red[wid * kSpec + lane] = f2_st(u);
      ered[wid * kSpec + lane] = err;
    }
    __syncthreads();
    if (threadIdx.x < na) {
      f2 s2 = f2_f(0.0f);
      int e = 0;
      for (int w = 0; w < kGrandWarps; ++w) {
        s2 = f2_add(s2, f2_ld(red[w * kSpec + threadIdx.x]));
        e |= ered[w * kSpec + threadIdx.x];
      }
      reinterpret_cast<float2 *>(p.ipart)[(size_t)blockIdx.x * kSpec + threadIdx.x] = f2_st(s2);
      p.ierr[(size_t)blockIdx.x * kSpec + threadIdx.x] = e;
    }
    __syncthreads();  // the partials, then the release of the arrival
    if (threadIdx.x == 0) release_add(&st->bar_count, 1u);
  }
  launch_exit(st);
}

// The widest GRAND grid at capacity cap: a lane per (particle, attempt) at
// the most attempts a round holds (kSpec, the fewest particles a block
// takes), the attempts' new slots, and the coordinator.
int grand_slots(int cap) {
  const int per_blk = kGrandWarps * (32 / kSpec);
  return (cap + kSpec + per_blk - 1) / per_blk + 1;
}

// Blocks of the GRAND launch: the coordinator and enough blocks for a lane
// per (particle, attempt of a round), all co-resident, at most the partial
// slots the context holds (ipart_slots, grand_slots of its capacity); with
// fewer, a lane takes several particles.
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
  KP pc = p;  // the barrier counters are zero between launches (launch_exit)
  void *args[] = {(void *)&pc, (void *)&mask, (void *)&seed, (void *)&cycle, (void *)&ngcmc,
                  (void *)&ffpos};
  return cudaLaunchCooperativeKernel((const void *)k_grand, dim3(grid), dim3(kGrandThreads),
                                     args, 0, stream);
}

// ---------------------------------------------------------------------------
// GRAND one attempt after another (grand.f90:19-121, insert.f90, find.f90
// as the reference runs them), for systems with a ΔE term the round kernel
// does not form: the MMIJ reaction field, which every ion feels through the
// basis coefficients.  Per attempt, in stream order:
//   k_gseq_propose  one block: the draws (propose_draws), a deletion's
//                   target by a block scan of the buffer tags in slot
//                   order; writes the trial;
//   INTERACT        launch_interact with its MMIJ term, a deletion trial
//                   counting its warnings;
//   k_gseq_accept   one thread: the acceptance draw and rule (accept_rate),
//                   the move on the FP64 arrays, prob(ib, nat(ib)) += 1.
// The draws and the rule are k_grand's, so on a system both can run the two
// make the same moves.
// ---------------------------------------------------------------------------
// The context's buffer parameters and counts as propose_draws / accept_rate
// read them.
struct KPBuf {
  int nbuf;
  const double *avnum, *mu, *kbb, *lzmin, *lzmax, *rmin, *rmax;
  const int *ibfftyp;
  const uint8_t *qbias;
  const int *nat, *ntotat;
};
__device__ __forceinline__ KPBuf kp_buf(const KP &p) {
  return KPBuf{p.nbuffer, p.avnum, p.mu, p.kbb, p.lzmin, p.lzmax, p.rmin, p.rmax,
               p.ibfftyp, p.qbufferbias, p.st->nat, p.st->ntotat};
}

constexpr int kGseqThreads = 256;

__global__ void __launch_bounds__(kGseqThreads)
    k_gseq_propose(KP p, uint64_t seed, uint64_t cycle, int a) {
  __shared__ Trial s_tr;
  __shared__ int s_rank, s_found, s_cnt[kGseqThreads / 32];
  const int tid = threadIdx.x;
  const int ntot = p.st->ntot;
  if (tid == 0) {
    Trial t;
    double u = 0.0;
    propose_draws(p, seed, cycle, (uint32_t)a, kp_buf(p), t, u);
    t.ntot = ntot;
    t.chg = -1;
    s_rank = 0;
    if (t.insert) {
      t.j = ntot + 1;
    } else {
      const int ib = t.ib;
      const int natb = ib <= p.nbuffer ? p.st->nat[ib - 1] : 0;
      const int ip = (int)((double)natb * u) + 1;
      t.valid = 0;
      if (ib <= p.nbuffer && ip <= natb) {
        t.itype = p.ibfftyp[ib];
        t.valid = 1;
        s_rank = ip;
      }
    }
    s_tr = t;
    s_found = -1;
  }
  __syncthreads();
  if (s_rank > 0) {  // find.f90: the s_rank-th ion of the buffer in slot order
    const int ib = s_tr.ib, rank = s_rank;
    int before = 0;
    for (int c0 = p.nsites + p.nfix; c0 < ntot && before < rank; c0 += kGseqThreads) {
      const int i = c0 + tid;
      const bool m = i < ntot && p.ibuffer[i] == ib;
      const unsigned bal = __ballot_sync(0xffffffffu, m);
      if ((tid & 31) == 0) s_cnt[tid >> 5] = __popc(bal);
      __syncthreads();
      int wb = 0, all = 0;
      for (int w = 0; w < kGseqThreads / 32; ++w) {
        if (w < (tid >> 5)) wb += s_cnt[w];
        all += s_cnt[w];
      }
      if (m && before + wb + __popc(bal & ((1u << (tid & 31)) - 1u)) + 1 == rank) s_found = i;
      before += all;  // the same on every thread: the loop ends together
      __syncthreads();
    }
    if (tid == 0) {
      const int k = s_found;
      if (k < 0 || guard_bad(p.st, k, ntot, 11)) {
        s_tr.valid = 0;
        atomicOr(&p.st->err, kErrFind);
      } else {
        s_tr.j = k + 1;
        s_tr.x = p.x[k];
        s_tr.y = p.y[k];
        s_tr.z = p.z[k];
      }
    }
  }
  __syncthreads();
  if (tid == 0) *p.trial = s_tr;
}

__global__ void k_gseq_accept(KP p, uint64_t seed, uint64_t cycle, int a, const double *de_dev) {
  if (threadIdx.x != 0) return;
  DevState *st = p.st;
  const Trial t = *p.trial;
  const int nb = p.nbuffer;
  if (t.valid && !guard_bad(st, t.ib - 1, nb, 21)) {
    const double de = *de_dev;
    const int ib = t.ib, b = ib - 1, nat = st->nat[b], ntot = st->ntot;
    const double rate = accept_rate(p, kp_buf(p), t, de, cycle);
    if (gcmc_uniform(seed, cycle, (uint32_t)a, (uint32_t)t.draw) <= rate) {
      if (t.insert) {
        if (ntot + 1 > p.cap) {
          atomicOr(&st->err, kErrCapacity);
        } else {
          p.x[ntot] = t.x;
          p.y[ntot] = t.y;
          p.z[ntot] = t.z;
          p.typei[ntot] = t.z < p.cz ? -t.itype : t.itype;
          p.ibuffer[ntot] = ib;
          st->nat[b] = nat + 1;
          st->ninsert[b] += 1;
          st->dener_sum += de;
          st->ntot = ntot + 1;
        }
      } else if (!guard_bad(st, t.j - 1, ntot, 23)) {
        const int iat = t.j - 1, last = ntot - 1;
        p.x[iat] = p.x[last];
        p.y[iat] = p.y[last];
        p.z[iat] = p.z[last];
        p.typei[iat] = p.typei[last];
        p.ibuffer[iat] = p.ibuffer[last];
        st->nat[b] = nat - 1;
        st->nremove[b] += 1;
        st->dener_sum -= de;
        st->ntot = ntot - 1;
      }
    }
  }
  for (int b = 0; b < nb; ++b) {  // grand.f90:117-119
    const int n = st->nat[b];
    if (!guard_bad(st, n, p.cap + 1, 25)) p.prob[(size_t)b * (p.cap + 1) + n] += 1;
  }
}

int launch_grand_seq(const KP &p, int ntot_ub, uint32_t mask, uint64_t seed, uint64_t cycle,
                     int ngcmc, double *de_dev, cudaStream_t stream) {
  cudaMemsetAsync(&p.st->dener_sum, 0, sizeof(double), stream);
  int nl = 0;
  for (int a = 0; a < ngcmc; ++a) {
    const int ub = std::min(p.cap, ntot_ub + a);  // each attempt adds at most one ion
    k_gseq_propose<<<1, kGseqThreads, 0, stream>>>(p, seed, cycle, a);
    launch_interact(p, ub, mask, -1, de_dev, stream);
    k_gseq_accept<<<1, 32, 0, stream>>>(p, seed, cycle, a, de_dev);
    nl += 5 + ((mask & 16u) && p.qrfpar ? 1 : 0) + ((mask & 64u) && p.mm.on ? 5 : 0);
  }
  return nl;
}

// ---------------------------------------------------------------------------
// COUNT (count.f90:19-95), once per cycle after the BD steps: each mobile
// ion's buffer -- the first whose ion type and z range (for a sphere also the
// radial shell) hold it --, nat by integer atomics (order-free, so exact), the
// sign of a buffer ion's type by its side of cz, then ntotat += nat.  A
// buffer ion outside the system (the reference's fatal error) raises
// kErrOutside.
// ---------------------------------------------------------------------------
// One particle's COUNT: its buffer (0 none); adds to nat[b - 1] and fixes
// the sign of its type.
template <bool FF>
__device__ __forceinline__ int count_one(const KP &p, int i, int *nat) {
  int ib = 0;
  if (i >= p.nsites + p.nfix) {
    const double3 q = pos_of(p, FF, i);
    const int itype = abs(p.typei[i]);
    for (int b = 1; b <= p.nbuffer && !ib; ++b) {
      if (itype != p.ibfftyp[b] || !(q.z >= p.lzmin[b] && q.z <= p.lzmax[b])) continue;
      bool out = false, in = true;
      if (p.shape == 1) {
        const double r2 = (q.x - p.cx) * (q.x - p.cx) + (q.y - p.cy) * (q.y - p.cy) +
                          (q.z - p.cz) * (q.z - p.cz);
        out = r2 > p.rsphe2;
        in = r2 >= p.rmin[b] * p.rmin[b] && r2 <= p.rmax[b] * p.rmax[b];
      } else {
        if (p.shape == 2) {
          const double ex = (q.x - p.cx) * p.iecx, ey = (q.y - p.cy) * p.iecy;
          out = ex * ex + ey * ey > 1.0;
        } else {
          out = q.x < p.lx2m || q.x > p.lx2p || q.y < p.ly2m || q.y > p.ly2p;
        }
        out = out || q.z < p.lz2m || q.z > p.lz2p;
      }
      if (out) atomicOr(&p.st->err, kErrOutside);
      if (!in) continue;
      ib = b;
      atomicAdd(&nat[b - 1], 1);
      p.typei[i] = q.z < p.cz ? -itype : itype;
    }
  }
  return ib;
}

// The whole COUNT in one launch over many blocks: the range tests are FP64
// (a few FP64 operations a clock per SM), so the particles are spread over
// the SMs.  Each block sums its nat in shared memory and adds it to
// DevState::count_acc; the last block to finish (a ticket after a fence)
// publishes nat, adds it to ntotat and clears the scratch for the next
// launch.  Integer sums: exact in any order.
constexpr int kCountThreads = 32;
template <bool FF>
__global__ void __launch_bounds__(kCountThreads) k_count_grid(KP p) {
  __shared__ int nat[kMaxBuffers];
  __shared__ bool last;
  for (int b = threadIdx.x; b < p.nbuffer; b += blockDim.x) nat[b] = 0;
  __syncthreads();
  const int ntot = p.st->ntot;
  for (int i = p.nsites + blockIdx.x * blockDim.x + threadIdx.x; i < ntot;
       i += gridDim.x * blockDim.x)
    p.ibuffer[i] = count_one<FF>(p, i, nat);
  __syncthreads();
  for (int b = threadIdx.x; b < p.nbuffer; b += blockDim.x)
    if (nat[b]) atomicAdd(&p.st->count_acc[b], nat[b]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&p.st->count_done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int b = threadIdx.x; b < p.nbuffer; b += blockDim.x) {
    const int v = atomicExch(&p.st->count_acc[b], 0);
    p.st->nat[b] = v;
    p.st->ntotat[b] += v;
  }
  if (threadIdx.x == 0) p.st->count_done = 0u;
}

int launch_count(const KP &p, bool ff, int ntot_ub, cudaStream_t stream) {
  if (p.nbuffer < 1) return 0;
  static int nsm[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (!nsm[dev] && cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev) !=
                       cudaSuccess)
    nsm[dev] = 1;
  const int n = std::max(1, ntot_ub - p.nsites);
  const int grid = std::max(1, std::min(nsm[dev], (n + kCountThreads - 1) / kCountThreads));
  (ff ? k_count_grid<true> : k_count_grid<false>)<<<grid, kCountThreads, 0, stream>>>(p);
  return 1;
}

// ---------------------------------------------------------------------------
// GRAND on every replica of a batch (grand.f90:19-121, insert.f90, find.f90):
// one block per replica, the attempts one after another as the reference
// makes them, each ΔE the FP64 INTERACT of the single context
// (trial_single_warp, interact_rec) over the replica's slots, positions read
// from the float-float records.  The draws are the single context's (the
// replica's seed, the cycle, the attempt), so a replica makes the moves
// bromoc_gpu_grand makes on a context holding it.  An accepted move rewrites
// the records in place: an insertion appends (records, type, buffer, RFPAR
// gathers), a deletion copies the last ion into the hole.
// ---------------------------------------------------------------------------
constexpr int kBgThreads = 256;

__global__ void __launch_bounds__(kBgThreads)
    k_batch_grand(KP p, const RepDev *rep, RepGc *gcs, int *ibuf, uint32_t mask,
                  const uint64_t *seeds, uint64_t cycle, int ngcmc) {
  __shared__ Trial tr;
  __shared__ int s_n, s_iat, s_acc, s_cnt[kBgThreads / 32];
  __shared__ double red[kBgThreads / 32], tot[1];
  const int r = blockIdx.x, tid = threadIdx.x;
  const RepDev R = rep[r];
  RepGc &G = gcs[r];
  const int off = R.off;
  const uint64_t seed = seeds[r];
  const bool rf_on = (mask & 16u) && p.qrfpar;
  if (tid == 0) {
    s_n = G.n;
    G.err = 0;
    G.dener = 0.0;
  }
  __syncthreads();
  // RFPAR gathers of the replica's ions at their positions (interact's cross term)
  if (rf_on)
    for (int i = tid; i < s_n; i += blockDim.x) {
      const double3 q = pos_of(p, true, off + i);
      p.gc_rf[off + i] = rf_single(p, q.x, q.y, q.z, abs(p.typei[off + i]));
    }
  __syncthreads();
  const int nb = G.nb;
  for (int a = 0; a < ngcmc; ++a) {
    const int n = s_n;
    if (tid == 0) {  // the draws: propose_draws with the replica's box and buffers
      Trial t{};
      Draws d{seed, cycle, (uint32_t)a};
      if (d.next() < 0.5) {
        const int ib = (int)((double)nb * d.next()) + 1;
        t.insert = 1;
        t.ib = ib;
        if (ib <= nb && G.buf[ib - 1].avnum > 0.0) {
          const RepBuf &B = G.buf[ib - 1];
          t.itype = B.ibfftyp;
          t.valid = 1;
          bool ok = false;
          for (int it = 0; it < (1 << 20) && !ok; ++it) {
            const double u1 = d.next(), u2 = d.next(), u3 = d.next();
            t.x = G.lx * (u1 - 0.5) + G.cx;
            t.y = G.ly * (u2 - 0.5) + G.cy;
            t.z = B.lzmin + (B.lzmax - B.lzmin) * u3;
            ok = true;
            if (G.shape == 1) {
              const double r2 = (t.x - G.cx) * (t.x - G.cx) + (t.y - G.cy) * (t.y - G.cy) +
                                (t.z - G.cz) * (t.z - G.cz);
              ok = r2 > B.rmin * B.rmin && r2 < B.rmax * B.rmax;
            } else if (G.shape == 2) {
              const double ex = (t.x - G.cx) * G.iecx, ey = (t.y - G.cy) * G.iecy;
              ok = ex * ex + ey * ey < 1.0;
            }
          }
          if (!ok) {
            t.valid = 0;
            G.err |= kErrFind;
          }
          t.j = off + n + 1;  // 1-based slot of the newcomer
          if (t.valid && n + 1 > R.cap) {
            t.valid = 0;
            G.err |= kErrCapacity;
          }
        }
      } else {
        t.ib = (int)((double)nb * d.next()) + 1;
        const double u_rank = d.next();
        t.insert = 0;
        const int natb = t.ib <= nb ? G.buf[t.ib - 1].nat : 0;
        const int ip = (int)((double)natb * u_rank) + 1;
        t.valid = t.ib <= nb && ip <= natb;
        s_iat = ip;  // the rank to find
      }
      t.draw = (int)d.n;
      tr = t;
    }
    __syncthreads();
    if (tr.valid && !tr.insert) {  // find.f90: the ip-th ion of the buffer in slot order
      const int ib = tr.ib, rank = s_iat;
      int before = 0, found = -1;
      for (int c0 = 0; c0 < n && found < 0; c0 += blockDim.x) {
        const int i = c0 + tid;
        const bool m = i < n && ibuf[off + i] == ib;
        const unsigned bal = __ballot_sync(0xffffffffu, m);
        if ((tid & 31) == 0) s_cnt[tid >> 5] = __popc(bal);
        __syncthreads();
        int wb = 0;
        for (int w = 0; w < (tid >> 5); ++w) wb += s_cnt[w];
        const int mine = before + wb + __popc(bal & ((1u << (tid & 31)) - 1u)) + 1;
        if (m && mine == rank) s_acc = i;
        int all = 0;
        for (int w = 0; w < kBgThreads / 32; ++w) all += s_cnt[w];
        __syncthreads();
        if (before < rank && rank <= before + all) found = s_acc;
        before += all;
      }
      if (tid == 0) {
        if (found < 0) {
          tr.valid = 0;
          G.err |= kErrFind;
        } else {
          const double3 q = pos_of(p, true, off + found);
          tr.j = off + found + 1;
          tr.itype = G.buf[ib - 1].ibfftyp;
          tr.x = q.x;
          tr.y = q.y;
          tr.z = q.z;
        }
      }
      __syncthreads();
    }
    if (!tr.valid) {  // block-uniform; every thread has read tr before it changes
      __syncthreads();
      continue;
    }
    if (tid < 32) {  // the single-particle terms (warnings not counted in a batch)
      Trial t = tr;
      int nalert = 0;
      trial_single_warp(p, t, mask, tr.insert ? 0 : 1, &nalert);
      __syncwarp();
      if (tid == 0) {
        tr.e_single = t.e_single;
        tr.srfe = t.srfe;
        tr.reff = t.reff;
        tr.rf_in = t.rf_in;
      }
    }
    __syncthreads();
    const Trial t = tr;
    const int jt2 = p.nwtype[t.itype];
    const bool rf = t.rf_in && rf_on;
    double u = 0.0;
    int err = 0;
    for (int i = tid; i < n; i += blockDim.x)
      if (off + i != t.j - 1) u += interact_rec(p, t, mask, off + i, jt2, true, rf,
                                                load_part(p, off + i, rf, true), err);
    if (err) atomicOr(&G.err, err);
    block_sum<1>(&u, red, tot);
    if (tid == 0) {  // acceptance (grand.f90:65-116) and the move
      const double de = t.e_single + tot[0];
      const RepBuf &B = G.buf[t.ib - 1];
      const double boltz = exp(-(de - B.mu) * p.ikbt);
      double rate;
      const int nat = B.nat;
      const double bias = B.avnum + B.kb * (B.avnum - (double)(B.ntotat / (long long)cycle));
      if (t.insert) {
        rate = B.qbias ? bias * boltz / (double)(nat + 1) : (B.avnum / (nat + 1)) * boltz;
        rate = rate / (1.0 + rate);
      } else {
        rate = B.qbias ? bias * boltz / (double)nat : (B.avnum / nat) * boltz;
        rate = 1.0 / (1.0 + rate);
      }
      Draws d{seed, cycle, (uint32_t)a};
      d.n = (uint32_t)t.draw;
      const bool acc = d.next() <= rate;
      RepBuf &W = G.buf[t.ib - 1];
      if (acc && t.insert) {
        const int s = off + n;
        const float xh = __double2float_rn(t.x), yh = __double2float_rn(t.y),
                    zh = __double2float_rn(t.z);
        const int code = (p.nwtype[t.itype] - 1) | (1 << 16);
        p.pk1[s] = make_float4(xh, yh, zh, __int_as_float(code));
        p.pk2[s] = make_float4(__double2float_rn(t.x - (double)xh),
                               __double2float_rn(t.y - (double)yh),
                               __double2float_rn(t.z - (double)zh), 0.0f);
        p.pk3[s] = make_float4(0.0f, (float)p.cg[t.itype], __int_as_float(2), 0.0f);
        p.typei[s] = t.z < G.cz ? -t.itype : t.itype;
        ibuf[s] = t.ib;
        if (rf_on) p.gc_rf[s] = rf ? make_double2(t.srfe, t.reff) : make_double2(0.0, 0.0);
        s_n = n + 1;
        W.nat += 1;
        W.ninsert += 1;
        G.dener += de;
      } else if (acc) {
        const int s = t.j - 1, l = off + n - 1;
        p.pk1[s] = p.pk1[l];
        p.pk2[s] = p.pk2[l];
        p.pk3[s] = p.pk3[l];
        p.typei[s] = p.typei[l];
        ibuf[s] = ibuf[l];
        if (rf_on) p.gc_rf[s] = p.gc_rf[l];
        s_n = n - 1;
        W.nat -= 1;
        W.nremove += 1;
        G.dener -= de;
      }
    }
    __syncthreads();
  }
  if (tid == 0) G.n = s_n;
}

// COUNT of every replica (count.f90 with the replica's box and buffers):
// one block per replica, nat by shared-memory integer atomics.
__global__ void __launch_bounds__(kBgThreads)
    k_batch_count(KP p, const RepDev *rep, RepGc *gcs, int *ibuf) {
  __shared__ int nat[kBatchMaxBuf], bad;
  const RepDev R = rep[blockIdx.x];
  RepGc &G = gcs[blockIdx.x];
  const int nb = G.nb;
  if (threadIdx.x < kBatchMaxBuf) nat[threadIdx.x] = 0;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < G.n; i += blockDim.x) {
    const int s = R.off + i;
    const double3 q = pos_of(p, true, s);
    const int itype = abs(p.typei[s]);
    int ib = 0;
    for (int b = 1; b <= nb && !ib; ++b) {
      const RepBuf &B = G.buf[b - 1];
      if (itype != B.ibfftyp || !(q.z >= B.lzmin && q.z <= B.lzmax)) continue;
      bool out = false, in = true;
      if (G.shape == 1) {
        const double r2 = (q.x - G.cx) * (q.x - G.cx) + (q.y - G.cy) * (q.y - G.cy) +
                          (q.z - G.cz) * (q.z - G.cz);
        out = r2 > G.rsphe2;
        in = r2 >= B.rmin * B.rmin && r2 <= B.rmax * B.rmax;
      } else {
        if (G.shape == 2) {
          const double ex = (q.x - G.cx) * G.iecx, ey = (q.y - G.cy) * G.iecy;
          out = ex * ex + ey * ey > 1.0;
        } else {
          out = q.x < G.cx - 0.5 * G.lx || q.x > G.cx + 0.5 * G.lx ||
                q.y < G.cy - 0.5 * G.ly || q.y > G.cy + 0.5 * G.ly;
        }
        out = out || q.z < G.cz - 0.5 * G.lz || q.z > G.cz + 0.5 * G.lz;
      }
      if (out) bad = 1;
      if (!in) continue;
      ib = b;
      atomicAdd(&nat[b - 1], 1);
      p.typei[s] = q.z < G.cz ? -itype : itype;
    }
    ibuf[s] = ib;
  }
  __syncthreads();
  if (threadIdx.x < nb) {
    G.buf[threadIdx.x].nat = nat[threadIdx.x];
    G.buf[threadIdx.x].ntotat += nat[threadIdx.x];
  }
  if (threadIdx.x == 0 && bad) G.err |= kErrOutside;
}

void launch_batch_count(const KP &p, const RepDev *rep, RepGc *gc, int *ibuf, int nrep,
                        cudaStream_t stream) {
  if (nrep > 0) k_batch_count<<<nrep, kBgThreads, 0, stream>>>(p, rep, gc, ibuf);
}

void launch_batch_grand(const KP &p, const RepDev *rep, RepGc *gc, int *ibuf, int nrep,
                        uint32_t mask, const uint64_t *seeds, uint64_t cycle, int ngcmc,
                        cudaStream_t stream) {
  if (nrep <= 0 || ngcmc <= 0) return;
  k_batch_grand<<<nrep, kBgThreads, 0, stream>>>(p, rep, gc, ibuf, mask, seeds, cycle, ngcmc);
}

}  // namespace bgpu
