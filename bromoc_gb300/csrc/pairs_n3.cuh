// The Newton-3 FP32 pair tile shared by the pair kernel and the fused BD
// loop kernel.
#pragma once
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"

#include <cuda/std/type_traits>

namespace bgpu {

// ---------------------------------------------------------------------------
// FP32 pair kernel with Newton's third law: each unordered ion pair once.
// Ions form tiles of 32; one warp takes tile pair (I, J), I <= J, from a
// flat row-major list.  Lane l holds row ion i = I*32 + l in registers; the
// column tile's records and its force accumulators sit in the warp's shared
// memory.  At step k lane l meets column lane m = (l + k) mod 32, so in one
// step the 32 lanes touch 32 different column entries and the column forces
// need no atomics (a __syncwarp orders the steps).  A diagonal tile uses
// k = 1..16, half of the lanes at k = 16, so each pair inside it appears once.
// Same laws and rules as k_pairs32 (ion-ion force only on mobile ions, the
// RFPAR chain on every ion in the map); the energy of a pair is added once.
// Records are read past L1 (__ldcg): in the fused BD loop other blocks
// wrote them earlier in the same launch.
// Output: per tile pair and side, per lane, (f, A) and B (tpf, tpb); the
// assembly kernel sums a particle's row and column entries in fixed order.
// ---------------------------------------------------------------------------
// Extension mode (periodic box): the nearest image of a separation whose
// components are at most one box length; rintf rounds half to even, as the
// FP64 path's rint.
__device__ __forceinline__ void min_image_f(const KP &p, float &dx, float &dy, float &dz) {
  dx = fmaf(-p.f.L[0], rintf(dx * p.f.iL[0]), dx);
  dy = fmaf(-p.f.L[1], rintf(dy * p.f.iL[1]), dy);
  dz = fmaf(-p.f.L[2], rintf(dz * p.f.iL[2]), dz);
}

// FP64 r^2 of a pair for srp_branch (the SRPMF boundary decision), with the
// nearest image in the periodic extension mode: the same whole-box shifts as
// min_image_f, in FP64 lengths as the FP64 path takes them.  The source's
// records are read again from the warp's shared arrays (entry mm): volatile
// reads, so that the pair loop need not keep them live for this rare path.
template <bool PBC>
__device__ __forceinline__ double pair_r2_64(const KP &p, const float4 &th, const float4 &tl,
                                             int mm, const float4 *sh, const float4 *sl) {
  const volatile float *vh = reinterpret_cast<const volatile float *>(sh + mm);
  const volatile float *vl = reinterpret_cast<const volatile float *>(sl + mm);
  const float4 h = make_float4(vh[0], vh[1], vh[2], 0.f);
  const float4 l = make_float4(vl[0], vl[1], vl[2], 0.f);
  if (!PBC) return r2_ff64(th, tl, h, l);
  const float dx = (th.x - h.x) + (tl.x - l.x), dy = (th.y - h.y) + (tl.y - l.y),
              dz = (th.z - h.z) + (tl.z - l.z);
  return r2_ff64(th, tl, h, l, p.lx * (double)rintf(dx * p.f.iL[0]),
                 p.ly * (double)rintf(dy * p.f.iL[1]), p.lz * (double)rintf(dz * p.f.iL[2]));
}

// Systems up to this many ion tiles run the pair tile's two-chain loop.
constexpr int kN3DualTiles = 96;

// Pair index of two particles' type codes (only on the rare SRPMF branch:
// the dense law table keeps the SRPMF cutoff, not the index).
__device__ __forceinline__ int srp_index(const KP &p, int code_i, int code_j) {
  return __ldg(p.pidx + (code_i & 0xffff) * p.nttyp + (code_j & 0xffff));
}

// The particle records and partial buffers of one system for the pair tile:
// a context's own arrays, or one replica's slots and partials in a batch.
struct PairSys {
  const float4 *pk1, *pk2, *pk3;
  float4 *tpf;
  float *tpb;
  int nsites, nfix;
  int ntot;  // live particles
  int T;     // ion tiles of 32
};

__device__ __forceinline__ PairSys pair_sys(const KP &p, int ntot, int T) {
  return PairSys{p.pk1, p.pk2, p.pk3, p.tpf, p.tpb, p.nsites, p.nfix, ntot, T};
}

// One tile pair q of the Newton-3 pair kernel, run by one warp (all 32
// lanes).  sh/sl/sq/acc/accb/acc1/accb1: the warp's own 32-entry shared
// arrays; tab:
// the block's dense ion-ion law table; e: the lane's energy sums (ecoul,
// elj, esrpmf, eefpot, erfpar), added to; without EFP the elj sum holds
// 6 x elj (the dense table holds 6 epp4).
// p: the laws and constants.
template <bool II, bool RF, bool EFP, bool PBC = false>
__device__ __forceinline__ void n3_tile(const KP &p, const PairSys &ps, int q, int qforces,
                                        float4 *sh, float4 *sl, float4 *sq, float4 *acc,
                                        float *accb, float4 *acc1, float *accb1,
                                        const float4 *tab, float e[5]) {
  const int lane = threadIdx.x & 31;
  const int nt = p.nion_t;
  const int T = ps.T, ntot = ps.ntot;
  const int m0 = ps.nsites + ps.nfix;
  float fx = 0.f, fy = 0.f, fz = 0.f, A = 0.f, B = 0.f;
  bool iv = false;
  int jl = 0;
  __syncwarp();  // the warp's arrays may still hold the previous tile pair
  // row I of q: the largest I with offset(I) <= q
  int I = (int)((2.0f * T + 1.0f - sqrtf((2.0f * T + 1.0f) * (2.0f * T + 1.0f) - 8.0f * q)) * 0.5f);
  I = max(0, min(I, T - 1));
  while (I > 0 && n3_index(T, I, I) > q) --I;
  while (I + 1 < T && n3_index(T, I + 1, I + 1) <= q) ++I;
  const int J = I + (q - n3_index(T, I, I));
  const bool diag = I == J;
  const int i = ps.nsites + I * 32 + lane;
  jl = ps.nsites + J * 32 + lane;
  // column tile into shared memory; its first ncol slots hold ions.  An
  // empty slot sits 1e10 A away with zero charge, srfe and reff and the first
  // ion type, so the branch-free path below can run over it with its law
  // entry zeroed: every term it adds is then exactly zero.
  const int ncol = min(32, max(0, ntot - (ps.nsites + J * 32)));
  if (jl < ntot) {
    sh[lane] = __ldcg(ps.pk1 + jl);
    sl[lane] = __ldcg(ps.pk2 + jl);
    if (RF) sq[lane] = __ldcg(ps.pk3 + jl);
  } else {
    sh[lane] = make_float4(1e10f, 1e10f, 1e10f, __int_as_float(EFP ? 0 : p.ndna));
    sl[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (RF) sq[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  acc[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  acc1[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (RF) accb[lane] = accb1[lane] = 0.f;
  iv = i < ntot;
  float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th, tq = th;
  if (iv) {
    th = __ldcg(ps.pk1 + i);
    tl = __ldcg(ps.pk2 + i);
    if (RF) tq = __ldcg(ps.pk3 + i);
  }
  const int tcode = __float_as_int(th.w);
  const bool tmob = iv && i >= m0;
  const int row = EFP ? (tcode & 0xffff) * p.nttyp : ((tcode & 0xffff) - p.ndna) * nt;
  const int tb = __float_as_int(tq.z);
  const float srt = tl.w, rft = tq.x, ct = p.f.celec * tq.y;
  __syncwarp();
  // Fast path: an off-diagonal tile pair whose 32 row ions are present and
  // whose ions are all mobile: no per-pair validity, mobility or role test.
  // With RFPAR every ion must either qualify for the cross term in both
  // roles (flags 4 and 8) or lie outside the RFPAR map (flag 1 clear), where
  // its srfe and reff are zero and every cross-term quantity of its pairs
  // comes out exactly zero.  A column tile with empty slots (RAG) zeroes
  // their law entries instead.
  bool lane_ok = iv && tmob && (jl >= ntot || jl >= m0);
  if (RF) {
    const int sb0 = __float_as_int(sq[lane].z);
    lane_ok = lane_ok && ((tb & 12) == 12 || !(tb & 1)) &&
              (jl >= ntot || (sb0 & 12) == 12 || !(sb0 & 1));
  }
  const bool fast = II && !EFP && !diag && __all_sync(0xffffffffu, lane_ok);
  // One pair of the branch-free loop: row lane against column entry mm, its
  // terms into the row sums (gx, gy, gz, gA, gB, ge) and into the column
  // sums ac[mm], acb[mm].
  auto pair_step = [&](auto rag, int mm, float4 *ac, float *acb, float &gx, float &gy,
                       float &gz, float &gA, float &gB, float *ge) {
    constexpr bool RAG = decltype(rag)::value;
    const float4 h = sh[mm], l = sl[mm];
    float dx = (th.x - h.x) + (tl.x - l.x);
    float dy = (th.y - h.y) + (tl.y - l.y);
    float dz = (th.z - h.z) + (tl.z - l.z);
    if (PBC) min_image_f(p, dx, dy, dz);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    float4 c = tab[row + (__float_as_int(h.w) & 0xffff) - p.ndna];
    if ((RAG && mm >= ncol) || (PBC && r2 >= p.f.rc2)) c = make_float4(0.f, 0.f, c.z, 0.f);
    const float ir = rsqrt_nz(r2), ir2 = ir * ir;
    const float cofo = c.x * ir;
    ge[0] += cofo;
    float d6 = c.z * ir2;
    d6 = d6 * d6 * d6;
    const float d12 = d6 * d6;
    ge[1] = fmaf(c.y, d12 - d6, ge[1]);
    float de = ir2 * fmaf(c.y, fmaf(2.0f, d12, -d6), cofo);
    if (r2 <= c.w)
      de += srpmf32(p, srp_index(p, tcode, __float_as_int(h.w)), r2, ir, 1.0f, ge,
                    srp_branch(p, r2, [&] { return pair_r2_64<PBC>(p, th, tl, mm, sh, sl); }));
    float4 a = ac[mm];
    if (RF) {
      const float4 u = sq[mm];
      const float rij = u.x * rft, srij = l.w * srt;
      const float rfdn = rsqrt_nz(fmaf(rij, rij, r2));
      const float aux0 = ct * u.y;
      const float a1 = aux0 * rij * rfdn;
      ge[4] = fmaf(a1, srij, ge[4]);
      const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
      const float aux3 = -a2 * fmaf(rij, 0.5f, r2);
      gA = fmaf(-a1, l.w, gA);
      gB = fmaf(aux3, u.x, gB);
      a.w = fmaf(-a1, srt, a.w);
      acb[mm] = fmaf(aux3, rft, acb[mm]);
      de = fmaf(a2, rij, de);
    }
    gx = fmaf(de, dx, gx);
    gy = fmaf(de, dy, gy);
    gz = fmaf(de, dz, gz);
    a.x = fmaf(-de, dx, a.x);
    a.y = fmaf(-de, dy, a.y);
    a.z = fmaf(-de, dz, a.z);
    ac[mm] = a;
  };
  // Two independent chains per step, k and k + 16, each with its own row
  // and column sums (acc / acc1): in one step both touch 32 distinct column
  // entries of their own arrays; the halves meet at the end.  Small systems
  // (T <= kN3DualTiles: about one tile pair per warp, latency-bound) take
  // it; larger ones, issue-bound, keep the single chain.  The choice depends
  // on T alone, so every kernel running a system of T tiles sums alike.
  auto fast_loop_dual = [&](auto rag) {
    float fx1 = 0.f, fy1 = 0.f, fz1 = 0.f, A1 = 0.f, B1 = 0.f;
    float e1[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < 16; ++k) {
      pair_step(rag, (lane + k) & 31, acc, accb, fx, fy, fz, A, B, e);
      pair_step(rag, (lane + k + 16) & 31, acc1, accb1, fx1, fy1, fz1, A1, B1, e1);
      __syncwarp();
    }
    fx += fx1;
    fy += fy1;
    fz += fz1;
    A += A1;
    B += B1;
#pragma unroll
    for (int m = 0; m < 5; ++m) e[m] += e1[m];
    const float4 a0 = acc[lane], a1 = acc1[lane];  // this lane's column entry
    acc[lane] = make_float4(a0.x + a1.x, a0.y + a1.y, a0.z + a1.z, a0.w + a1.w);
    if (RF) accb[lane] += accb1[lane];
  };
  auto fast_loop = [&](auto rag) {
    for (int k = 0; k < 32; ++k) {
      pair_step(rag, (lane + k) & 31, acc, accb, fx, fy, fz, A, B, e);
      __syncwarp();
    }
  };
  if (fast) {
    if (T <= kN3DualTiles) {
      if (ncol < 32)
        fast_loop_dual(cuda::std::true_type{});
      else
        fast_loop_dual(cuda::std::false_type{});
    } else {
      if (ncol < 32)
        fast_loop(cuda::std::true_type{});
      else
        fast_loop(cuda::std::false_type{});
    }
  } else {
    const int k0 = diag ? 1 : 0, k1 = diag ? 16 : 31;
    for (int k = k0; k <= k1; ++k) {
      const int mm = (lane + k) & 31;
      const float4 h = sh[mm];
      const int scode = __float_as_int(h.w);
      if (iv && mm < ncol && !(diag && k == 16 && lane >= 16)) {
        const float4 l = sl[mm];
        const int j = ps.nsites + J * 32 + mm;
        const bool smob = j >= m0;
        float dx = (th.x - h.x) + (tl.x - l.x);
        float dy = (th.y - h.y) + (tl.y - l.y);
        float dz = (th.z - h.z) + (tl.z - l.z);
        if (PBC) min_image_f(p, dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        float dii = 0.0f, drf = 0.0f, dAs = 0.0f, dBs = 0.0f;
        if (II && (tmob || smob) && !(PBC && r2 >= p.f.rc2)) {
          if (EFP) {
            dii = law32k(p, __ldg(p.pidx + row + (scode & 0xffff)), r2, 1.0f, e,
                         [&] { return pair_r2_64<PBC>(p, th, tl, mm, sh, sl); });
          } else {
            const float4 c = tab[row + (scode & 0xffff) - p.ndna];
            const float ir = rsqrt_nz(r2), ir2 = ir * ir;
            const float cofo = c.x * ir;
            e[0] += cofo;
            float d6 = c.z * ir2;
            d6 = d6 * d6 * d6;
            const float d12 = d6 * d6;
            e[1] = fmaf(c.y, d12 - d6, e[1]);
            dii = ir2 * fmaf(c.y, fmaf(2.0f, d12, -d6), cofo);
            if (r2 <= c.w)
              dii += srpmf32(p, srp_index(p, tcode, scode), r2, ir, 1.0f, e,
                             srp_branch(p, r2, [&] { return pair_r2_64<PBC>(p, th, tl, mm, sh, sl); }));
          }
        }
        if (RF) {
          const float4 sqv = sq[mm];
          const int sb = __float_as_int(sqv.z);
          if (i > j ? ((tb & 4) && (sb & 8)) : ((sb & 4) && (tb & 8))) {
            const float rij = sqv.x * rft, srij = l.w * srt;
            const float rfdn = rsqrt_nz(fmaf(rij, rij, r2));
            const float aux0 = ct * sqv.y;
            const float a1 = aux0 * rij * rfdn;
            e[4] = fmaf(a1, srij, e[4]);
            const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
            const float aux3 = -a2 * fmaf(rij, 0.5f, r2);
            A = fmaf(-a1, l.w, A);
            B = fmaf(aux3, sqv.x, B);
            dAs = -a1 * srt;
            dBs = aux3 * rft;
            drf = a2 * rij;
          }
        }
        const float dt = (tmob ? dii : 0.0f) + drf, ds = (smob ? dii : 0.0f) + drf;
        fx = fmaf(dt, dx, fx);
        fy = fmaf(dt, dy, fy);
        fz = fmaf(dt, dz, fz);
        float4 a = acc[mm];
        a.x = fmaf(-ds, dx, a.x);
        a.y = fmaf(-ds, dy, a.y);
        a.z = fmaf(-ds, dz, a.z);
        a.w += dAs;
        acc[mm] = a;
        if (RF) accb[mm] += dBs;
      }
      __syncwarp();
    }
  }
  // row side (lane l = row ion), column side (lane l = column ion)
  float4 *o = ps.tpf + (size_t)q * 64;
  o[lane] = qforces && iv ? make_float4(fx, fy, fz, A) : make_float4(0.f, 0.f, 0.f, 0.f);
  o[32 + lane] = qforces && jl < ntot ? acc[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
  if (RF) {
    float *ob = ps.tpb + (size_t)q * 64;
    ob[lane] = qforces && iv ? B : 0.f;
    ob[32 + lane] = qforces && jl < ntot ? accb[lane] : 0.f;
  }
}

}  // namespace bgpu
