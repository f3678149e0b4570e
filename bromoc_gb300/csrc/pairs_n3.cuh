// The Newton-3 FP32 pair tile shared by the pair kernel, the fused BD loop
// kernel and the replica-batch pair kernel.
#pragma once
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

// ---------------------------------------------------------------------------
// FP32 pair tile with Newton's third law: each unordered ion pair once.
// Ions form tiles of 32; one warp takes tile pair (I, J), I <= J, from a
// flat row-major list.  Lane l holds row ion i = I*32 + l in registers; the
// column tile's records and its force sums sit in the warp's shared memory.
// Same laws and rules as k_pairs32 (ion-ion force only on mobile ions, the
// RFPAR chain on every ion in the map); the energy of a pair is added once.
// Records are read past L1 (__ldcg): in the fused BD loop other blocks
// wrote them earlier in the same launch.
//
// Fast loop (off-diagonal tile pairs of mobile ions, analytic laws): at step
// k = 0..15 lane l meets column entries m = (l + k) mod 32 and m ^ 16 at
// once, as the two halves of packed f32x2 arithmetic (one instruction per
// operation for both pairs).  The column tile is stored in slots: slot m
// holds the fields of entries m and m ^ 16 side by side, and the column
// sums of slot m are those of entry m for the first half and of entry m ^ 16
// for the second.  In one step the 32 lanes touch 32 distinct slots, so the
// column sums need no atomics (a __syncwarp orders the steps); entry m's sum
// is slot m's first half plus slot m ^ 16's second half.
//
// SRPMF pairs (r^2 within the law's cutoff) are queued per warp and
// evaluated after the loop, 32 at a time, by lanes in parallel; their forces
// are then added in queue order (deterministic).  This keeps the rare SRPMF
// code -- exponential, sine and cosine, the FP64 boundary decision of
// srp_branch -- out of the loop's registers and its divergence.
//
// An empty column slot (a ragged last tile) sits 1e10 A away with zero
// charge, srfe and reff and points at the law table's zero column, so every
// term it adds is exactly zero and the loop needs no per-pair test.
//
// Sign conventions inside the tile: column sums and the A, B sums of the
// RFPAR chain are kept with the opposite sign and negated at the output.
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
// min_image_f, in FP64 lengths as the FP64 path takes them.
template <bool PBC>
__device__ __forceinline__ double pair_r2_64(const KP &p, const float4 &th, const float4 &tl,
                                             const float4 &h, const float4 &l) {
  if (!PBC) return r2_ff64(th, tl, h, l);
  const float dx = (th.x - h.x) + (tl.x - l.x), dy = (th.y - h.y) + (tl.y - l.y),
              dz = (th.z - h.z) + (tl.z - l.z);
  return r2_ff64(th, tl, h, l, p.lx * (double)rintf(dx * p.f.iL[0]),
                 p.ly * (double)rintf(dy * p.f.iL[1]), p.lz * (double)rintf(dz * p.f.iL[2]));
}

// Pair index of two particles' type codes (only on the rare SRPMF branch:
// the dense law table keeps the SRPMF cutoff, not the index).
__device__ __forceinline__ int srp_index(const KP &p, int code_i, int code_j) {
  return __ldg(p.pidx + (code_i & 0xffff) * p.nttyp + (code_j & 0xffff));
}

// SRPMF queue of a warp: entries a step can add at most (2 x 32), capacity.
constexpr int kSrpStep = 64;
constexpr int kSrpQ = 2 * kSrpStep;

// The warp's shared arrays of the pair tile.  Slot m (see above): p0 =
// (x hi of m, of m^16, y hi of m, of m^16), p1 = (z hi, z hi', x lo, x lo'),
// p2 = (y lo, y lo', z lo, z lo'), p3 = (law column, law column', srfe,
// srfe') with the law column as int bits, p4 = (reff, reff', charge,
// charge'); a0 = (fx, fx', fy, fy'), a1 = (fz, fz', A, A'), ab = (B, B').
// code / cflag: entry m's type code and RFPAR flags; q: the SRPMF queue
// (row lane | column entry << 5).
template <bool RF>
struct N3Warp {
  float4 p0[32], p1[32], p2[32], p3[32];
  float4 p4[RF ? 32 : 1];
  float4 a0[32], a1[32];
  float2 ab[RF ? 32 : 1];
  int code[32], cflag[RF ? 32 : 1];
  int q[kSrpQ];
};

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

// Entry m's position records from its slot (first halves).
template <bool RF>
__device__ __forceinline__ void n3_entry(const N3Warp<RF> &w, int m, float4 &h, float4 &l) {
  const float4 P0 = w.p0[m], P1 = w.p1[m], P2 = w.p2[m], P3 = w.p3[m];
  h = make_float4(P0.x, P0.z, P1.x, 0.f);
  l = make_float4(P1.z, P2.x, P2.z, P3.z);
}

// One tile pair q of the Newton-3 pair kernel, run by one warp (all 32
// lanes).  w: the warp's shared arrays; tab: the block's dense ion-ion law
// table (rows of ipq_stride(nt)); e: the lane's energy sums (ecoul, elj,
// esrpmf, eefpot, erfpar), added to; without EFP the elj sum holds 6 x elj
// (the dense table holds 6 epp4).  p: the laws and constants.
template <bool II, bool RF, bool EFP, bool PBC = false>
__device__ __forceinline__ void n3_tile(const KP &p, const PairSys &ps, int q, int qforces,
                                        N3Warp<RF> &w, const float4 *tab, float e[5]) {
  constexpr unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nt = p.nion_t;
  const int T = ps.T, ntot = ps.ntot;
  const int m0 = ps.nsites + ps.nfix;
  __syncwarp();  // the warp's arrays may still hold the previous tile pair
  // row I of q: the largest I with offset(I) <= q
  int I = (int)((2.0f * T + 1.0f - sqrtf((2.0f * T + 1.0f) * (2.0f * T + 1.0f) - 8.0f * q)) * 0.5f);
  I = max(0, min(I, T - 1));
  while (I > 0 && n3_index(T, I, I) > q) --I;
  while (I + 1 < T && n3_index(T, I + 1, I + 1) <= q) ++I;
  const int J = I + (q - n3_index(T, I, I));
  const bool diag = I == J;
  const int i = ps.nsites + I * 32 + lane;
  const int jl = ps.nsites + J * 32 + lane;
  const int ncol = min(32, max(0, ntot - (ps.nsites + J * 32)));
  // column entry `lane` into the slots (its own as the first half of slot
  // lane, as the second half of slot lane ^ 16)
  float4 h = make_float4(1e10f, 1e10f, 1e10f, __int_as_float(EFP ? 0 : p.ndna));
  float4 l = make_float4(0.f, 0.f, 0.f, 0.f), u = l;
  if (jl < ntot) {
    h = __ldcg(ps.pk1 + jl);
    l = __ldcg(ps.pk2 + jl);
    if (RF) u = __ldcg(ps.pk3 + jl);
  }
  const int hcode = __float_as_int(h.w);
  const int lcol = EFP ? 0 : (jl < ntot ? (hcode & 0xffff) - p.ndna : nt);
  {
    const float hx = __shfl_xor_sync(kAll, h.x, 16), hy = __shfl_xor_sync(kAll, h.y, 16),
                hz = __shfl_xor_sync(kAll, h.z, 16), lx = __shfl_xor_sync(kAll, l.x, 16),
                ly = __shfl_xor_sync(kAll, l.y, 16), lz = __shfl_xor_sync(kAll, l.z, 16),
                lw = __shfl_xor_sync(kAll, l.w, 16);
    const int lc = __shfl_xor_sync(kAll, lcol, 16);
    w.p0[lane] = make_float4(h.x, hx, h.y, hy);
    w.p1[lane] = make_float4(h.z, hz, l.x, lx);
    w.p2[lane] = make_float4(l.y, ly, l.z, lz);
    w.p3[lane] = make_float4(__int_as_float(lcol), __int_as_float(lc), l.w, lw);
    if (RF) {
      const float ux = __shfl_xor_sync(kAll, u.x, 16), uy = __shfl_xor_sync(kAll, u.y, 16);
      w.p4[lane] = make_float4(u.x, ux, u.y, uy);
      w.ab[lane] = make_float2(0.f, 0.f);
      w.cflag[lane] = __float_as_int(u.z);
    }
    w.a0[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.a1[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.code[lane] = hcode;
  }
  const bool iv = i < ntot;
  float4 th = make_float4(0.f, 0.f, 0.f, 0.f), tl = th, tq = th;
  if (iv) {
    th = __ldcg(ps.pk1 + i);
    tl = __ldcg(ps.pk2 + i);
    if (RF) tq = __ldcg(ps.pk3 + i);
  }
  const int tcode = __float_as_int(th.w);
  const bool tmob = iv && i >= m0;
  const int row = EFP ? (tcode & 0xffff) * p.nttyp : ((tcode & 0xffff) - p.ndna) * ipq_stride(nt);
  const int tb = __float_as_int(tq.z);
  const float srt = tl.w, rft = tq.x, ct = p.f.celec * tq.y;
  // row sums: two halves in the fast loop, the first alone elsewhere
  float2 FX = v2(0.f), FY = v2(0.f), FZ = v2(0.f), NA = v2(0.f), NB = v2(0.f);
  float2 E0 = v2(0.f), E1 = v2(0.f), E4 = v2(0.f);
  // Fast loop: an off-diagonal tile pair whose 32 row ions are present and
  // whose ions are all mobile: no per-pair validity, mobility or role test.
  // With RFPAR every ion must either qualify for the cross term in both
  // roles (flags 4 and 8) or lie outside the RFPAR map (flag 1 clear), where
  // its srfe and reff are zero and every cross-term quantity of its pairs
  // comes out exactly zero.
  bool lane_ok = iv && tmob && (jl >= ntot || jl >= m0);
  if (RF) {
    const int sb0 = __float_as_int(u.z);
    lane_ok = lane_ok && ((tb & 12) == 12 || !(tb & 1)) &&
              (jl >= ntot || (sb0 & 12) == 12 || !(sb0 & 1));
  }
  const bool fast = II && !EFP && !diag && __all_sync(kAll, lane_ok);
  __syncwarp();
  if (fast) {
    const float2 THX = v2(th.x), THY = v2(th.y), THZ = v2(th.z);
    const float2 TLX = v2(tl.x), TLY = v2(tl.y), TLZ = v2(tl.z);
    const float2 SRT = v2(srt), RFT = v2(rft), CT = v2(ct);
    const float4 *tr = tab + row;
    const unsigned below = (1u << lane) - 1u;
    int qn = 0;  // queued SRPMF pairs (warp-uniform)
    auto srp_flush = [&]() {  // warp-uniform
      for (int b = 0; b < qn; b += 32) {
        const int idx = b + lane;
        const bool act = idx < qn;
        const int ent = act ? w.q[idx] : 0;
        const int r = ent & 31, j = ent >> 5;
        const float rhx = __shfl_sync(kAll, th.x, r), rhy = __shfl_sync(kAll, th.y, r),
                    rhz = __shfl_sync(kAll, th.z, r), rlx = __shfl_sync(kAll, tl.x, r),
                    rly = __shfl_sync(kAll, tl.y, r), rlz = __shfl_sync(kAll, tl.z, r);
        const int rcode = __shfl_sync(kAll, tcode, r);
        float gx = 0.f, gy = 0.f, gz = 0.f;
        if (act) {
          float4 ch, cl;
          n3_entry(w, j, ch, cl);
          // the r^2 of the loop, operation for operation
          float dx = (rhx - ch.x) + (rlx - cl.x);
          float dy = (rhy - ch.y) + (rly - cl.y);
          float dz = (rhz - ch.z) + (rlz - cl.z);
          if (PBC) min_image_f(p, dx, dy, dz);
          const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          const float4 rh = make_float4(rhx, rhy, rhz, 0.f), rl = make_float4(rlx, rly, rlz, 0.f);
          const float ds =
              srpmf32(p, srp_index(p, rcode, w.code[j]), r2, rsqrt_nz(r2), 1.0f, e,
                      srp_branch(p, r2, [&] { return pair_r2_64<PBC>(p, rh, rl, ch, cl); }));
          gx = ds * dx;
          gy = ds * dy;
          gz = ds * dz;
        }
        const int nb = min(32, qn - b);
        for (int t = 0; t < nb; ++t) {  // queue order
          const int rt = __shfl_sync(kAll, r, t), jt = __shfl_sync(kAll, j, t);
          const float vx = __shfl_sync(kAll, gx, t), vy = __shfl_sync(kAll, gy, t),
                      vz = __shfl_sync(kAll, gz, t);
          if (lane == rt) {
            FX.x += vx;
            FY.x += vy;
            FZ.x += vz;
            float4 a = w.a0[jt];
            a.x += vx;
            a.z += vy;
            w.a0[jt] = a;
            w.a1[jt].x += vz;
          }
          __syncwarp();
        }
      }
      qn = 0;
    };
#pragma unroll 2
    for (int k = 0; k < 16; ++k) {
      const int m = (lane + k) & 31;
      const float4 P0 = w.p0[m], P1 = w.p1[m], P2 = w.p2[m], P3 = w.p3[m];
      float2 dx = v2add(v2sub(THX, v2(P0.x, P0.y)), v2sub(TLX, v2(P1.z, P1.w)));
      float2 dy = v2add(v2sub(THY, v2(P0.z, P0.w)), v2sub(TLY, v2(P2.x, P2.y)));
      float2 dz = v2add(v2sub(THZ, v2(P1.x, P1.y)), v2sub(TLZ, v2(P2.z, P2.w)));
      if (PBC) {
        min_image_f(p, dx.x, dy.x, dz.x);
        min_image_f(p, dx.y, dy.y, dz.y);
      }
      const float2 r2 = v2fma(dx, dx, v2fma(dy, dy, v2mul(dz, dz)));
      float4 c0 = tr[__float_as_int(P3.x)], c1 = tr[__float_as_int(P3.y)];
      if (PBC) {
        if (r2.x >= p.f.rc2) c0 = make_float4(0.f, 0.f, 0.f, -1.f);
        if (r2.y >= p.f.rc2) c1 = make_float4(0.f, 0.f, 0.f, -1.f);
      }
      const float2 ir = v2(rsqrt_nz(r2.x), rsqrt_nz(r2.y));
      const float2 ir2 = v2mul(ir, ir);
      const float2 cofo = v2mul(v2(c0.x, c1.x), ir);
      E0 = v2add(E0, cofo);
      float2 d6 = v2mul(v2(c0.z, c1.z), ir2);
      d6 = v2mul(v2mul(d6, d6), d6);
      const float2 d12 = v2mul(d6, d6);
      const float2 t = v2sub(d12, d6);  // d12 - d6; d12 + t = 2 d12 - d6
      const float2 ce = v2(c0.y, c1.y);
      E1 = v2fma(ce, t, E1);
      float2 de = v2mul(ir2, v2fma(ce, v2add(d12, t), cofo));
      // SRPMF pairs into the queue, in (step, half, lane) order
      const bool s0 = r2.x <= c0.w, s1 = r2.y <= c1.w;
      const unsigned b0 = __ballot_sync(kAll, s0), b1 = __ballot_sync(kAll, s1);
      if (b0 | b1) {
        if (s0) w.q[qn + __popc(b0 & below)] = lane | (m << 5);
        if (s1) w.q[qn + __popc(b0) + __popc(b1 & below)] = lane | ((m ^ 16) << 5);
        qn += __popc(b0) + __popc(b1);
      }
      float2 a1 = v2(0.f), a2p = v2(0.f);
      if (RF) {
        const float4 P4 = w.p4[m];
        const float2 reff = v2(P4.x, P4.y), srfe = v2(P3.z, P3.w);
        const float2 rij = v2mul(reff, RFT), srij = v2mul(srfe, SRT);
        const float2 tt = v2fma(rij, rij, r2);
        const float2 rfdn = v2(rsqrt_nz(tt.x), rsqrt_nz(tt.y));
        const float2 aux0 = v2mul(CT, v2(P4.z, P4.w));
        a1 = v2mul(v2mul(aux0, rij), rfdn);
        E4 = v2fma(a1, srij, E4);
        const float2 a2 = v2mul(v2mul(v2mul(v2mul(aux0, srij), rfdn), rfdn), rfdn);
        a2p = v2mul(a2, v2fma(rij, v2(0.5f), r2));
        NA = v2fma(a1, srfe, NA);
        NB = v2fma(a2p, reff, NB);
        de = v2fma(a2, rij, de);
      }
      FX = v2fma(de, dx, FX);
      FY = v2fma(de, dy, FY);
      FZ = v2fma(de, dz, FZ);
      const float4 A0 = w.a0[m], A1 = w.a1[m];
      const float2 cx = v2fma(de, dx, v2(A0.x, A0.y)), cy = v2fma(de, dy, v2(A0.z, A0.w));
      const float2 cz = v2fma(de, dz, v2(A1.x, A1.y));
      const float2 ca = RF ? v2fma(a1, SRT, v2(A1.z, A1.w)) : v2(A1.z, A1.w);
      w.a0[m] = make_float4(cx.x, cx.y, cy.x, cy.y);
      w.a1[m] = make_float4(cz.x, cz.y, ca.x, ca.y);
      if (RF) w.ab[m] = v2fma(a2p, RFT, w.ab[m]);
      __syncwarp();
      if (qn > kSrpQ - kSrpStep) srp_flush();
    }
    if (qn) srp_flush();
  } else {
    const int k0 = diag ? 1 : 0, k1 = diag ? 16 : 31;
    for (int k = k0; k <= k1; ++k) {
      const int mm = (lane + k) & 31;
      if (iv && mm < ncol && !(diag && k == 16 && lane >= 16)) {
        float4 hc, lc;
        n3_entry(w, mm, hc, lc);
        const int scode = w.code[mm];
        const int j = ps.nsites + J * 32 + mm;
        const bool smob = j >= m0;
        float dx = (th.x - hc.x) + (tl.x - lc.x);
        float dy = (th.y - hc.y) + (tl.y - lc.y);
        float dz = (th.z - hc.z) + (tl.z - lc.z);
        if (PBC) min_image_f(p, dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        auto r2d = [&] { return pair_r2_64<PBC>(p, th, tl, hc, lc); };
        float dii = 0.0f, drf = 0.0f, dAs = 0.0f, dBs = 0.0f;
        if (II && (tmob || smob) && !(PBC && r2 >= p.f.rc2)) {
          if (EFP) {
            dii = law32k(p, __ldg(p.pidx + row + (scode & 0xffff)), r2, 1.0f, e, r2d);
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
                             srp_branch(p, r2, r2d));
          }
        }
        if (RF) {
          const float4 P4 = w.p4[mm];
          const int sb = w.cflag[mm];
          if (i > j ? ((tb & 4) && (sb & 8)) : ((sb & 4) && (tb & 8))) {
            const float rij = P4.x * rft, srij = lc.w * srt;
            const float rfdn = rsqrt_nz(fmaf(rij, rij, r2));
            const float aux0 = ct * P4.z;
            const float a1 = aux0 * rij * rfdn;
            e[4] = fmaf(a1, srij, e[4]);
            const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
            const float a2p = a2 * fmaf(rij, 0.5f, r2);
            NA.x = fmaf(a1, lc.w, NA.x);
            NB.x = fmaf(a2p, P4.x, NB.x);
            dAs = a1 * srt;
            dBs = a2p * rft;
            drf = a2 * rij;
          }
        }
        const float dt = (tmob ? dii : 0.0f) + drf, ds = (smob ? dii : 0.0f) + drf;
        FX.x = fmaf(dt, dx, FX.x);
        FY.x = fmaf(dt, dy, FY.x);
        FZ.x = fmaf(dt, dz, FZ.x);
        float4 a = w.a0[mm];
        a.x = fmaf(ds, dx, a.x);
        a.z = fmaf(ds, dy, a.z);
        w.a0[mm] = a;
        float4 b = w.a1[mm];
        b.x = fmaf(ds, dz, b.x);
        b.z += dAs;
        w.a1[mm] = b;
        if (RF) w.ab[mm].x += dBs;
      }
      __syncwarp();
    }
  }
  e[0] += E0.x + E0.y;
  e[1] += E1.x + E1.y;
  e[4] += E4.x + E4.y;
  // row side (lane l = row ion), column side (lane l = column entry l: the
  // first half of slot l plus the second half of slot l ^ 16)
  const float4 X0 = w.a0[lane], Y0 = w.a0[lane ^ 16], X1 = w.a1[lane], Y1 = w.a1[lane ^ 16];
  float4 *o = ps.tpf + (size_t)q * 64;
  o[lane] = qforces && iv ? make_float4(FX.x + FX.y, FY.x + FY.y, FZ.x + FZ.y, -(NA.x + NA.y))
                          : make_float4(0.f, 0.f, 0.f, 0.f);
  o[32 + lane] = qforces && jl < ntot
                     ? make_float4(-(X0.x + Y0.y), -(X0.z + Y0.w), -(X1.x + Y1.y), -(X1.z + Y1.w))
                     : make_float4(0.f, 0.f, 0.f, 0.f);
  if (RF) {
    float *ob = ps.tpb + (size_t)q * 64;
    ob[lane] = qforces && iv ? -(NB.x + NB.y) : 0.f;
    ob[32 + lane] = qforces && jl < ntot ? -(w.ab[lane].x + w.ab[lane ^ 16].y) : 0.f;
  }
}

}  // namespace bgpu
