// The Newton-3 FP32 pair tile shared by the pair kernel, the fused BD loop
// kernel and the replica-batch pair kernel.
#pragma once
#include "ff.cuh"
#include "launch.h"
#include "physics.cuh"

namespace bgpu {

// ---------------------------------------------------------------------------
// FP32 pair tile with Newton's third law: each unordered ion pair once.
// Ions form tiles of 32; one warp takes a work item (n3_item): a column
// tile J against one or two row tiles I < J (two: 64 row ions), or the
// diagonal tile pair (J, J).  Lane l holds row ion I*32 + l of each row tile
// in registers; the column tile's records and its force sums sit in the
// warp's shared memory, so with two row tiles each column read and each
// update of a column sum serves twice the pairs.
// Same laws and rules as k_pairs32 (ion-ion force only on mobile ions, the
// RFPAR chain on every ion in the map); the energy of a pair is added once.
// Records are read past L1 (__ldcg): in the fused BD loop other blocks
// wrote them earlier in the same launch.
//
// Fast loop (off-diagonal tile pairs of mobile ions, analytic laws): at step
// k = 0..15 lane l meets column entries m = (l + k) mod 32 and m ^ 16 at
// once, as the two halves of packed f32x2 arithmetic (one instruction per
// operation for both pairs), for each of the item's row tiles.  The column tile is stored in slots: slot m
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
// Every tile pair's entries are written by its item each pass.
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

// SRPMF queue of a warp: room for two steps of the two-row fast loop (each
// adds at most 4 x 32 entries).
constexpr int kSrpQ = 256;

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
  int rows;  // row tiles per work item: 2 (n3_item) or 1 (n3_pair)
};

__device__ __forceinline__ PairSys pair_sys(const KP &p, int ntot, int T, int rows) {
  return PairSys{p.pk1, p.pk2, p.pk3, p.tpf, p.tpb, p.nsites, p.nfix, ntot, T, rows};
}

// Entry m's position records from its slot (first halves).
template <bool RF>
__device__ __forceinline__ void n3_entry(const N3Warp<RF> &w, int m, float4 &h, float4 &l) {
  const float4 P0 = w.p0[m], P1 = w.p1[m], P2 = w.p2[m], P3 = w.p3[m];
  h = make_float4(P0.x, P0.z, P1.x, 0.f);
  l = make_float4(P1.z, P2.x, P2.z, P3.z);
}

// Lane l's row ion of one row tile of an item: records and the fields the
// tile reads.
struct N3Row {
  float4 th, tl;
  int i;      // particle
  int tcode;  // type code
  int row;    // offset of the ion's row in the law table
  int tb;     // RFPAR flags
  float srt, rft, ct;
  bool iv, tmob;  // present; mobile
};

// Row sums of one row tile: two halves in the fast loop, the first alone
// elsewhere; na, nb: the RFPAR chain's A and B sums (opposite sign).
struct N3Sum {
  float2 fx, fy, fz, na, nb;
};

template <bool RF, bool EFP>
__device__ __forceinline__ N3Row n3_row(const KP &p, const PairSys &ps, int I) {
  N3Row r;
  r.i = ps.nsites + I * 32 + (threadIdx.x & 31);
  r.iv = r.i < ps.ntot;
  float4 tq = make_float4(0.f, 0.f, 0.f, 0.f);
  r.th = tq;
  r.tl = tq;
  if (r.iv) {
    r.th = __ldcg(ps.pk1 + r.i);
    r.tl = __ldcg(ps.pk2 + r.i);
    if (RF) tq = __ldcg(ps.pk3 + r.i);
  }
  r.tcode = __float_as_int(r.th.w);
  r.tmob = r.iv && r.i >= ps.nsites + ps.nfix;
  r.row = EFP ? (r.tcode & 0xffff) * p.nttyp
              : ((r.tcode & 0xffff) - p.ndna) * ipq_stride(p.nion_t);
  r.tb = __float_as_int(tq.z);
  r.srt = r.tl.w;
  r.rft = tq.x;
  r.ct = p.f.celec * tq.y;
  return r;
}

// The fast loop's condition on a row ion: present and mobile; with RFPAR
// either qualified for the cross term in both roles (flags 4 and 8) or
// outside the RFPAR map (flag 1 clear), where its srfe and reff are zero and
// every cross-term quantity of its pairs comes out exactly zero.
template <bool RF>
__device__ __forceinline__ bool n3_row_fast(const N3Row &r) {
  return r.iv && r.tmob && (!RF || (r.tb & 12) == 12 || !(r.tb & 1));
}

// Column tile J into the warp's slots: entry `lane` as the first half of
// slot lane and the second half of slot lane ^ 16, column sums cleared.
// Returns the fast loop's condition on the lane's column entry (absent, or
// as n3_row_fast).
template <bool RF, bool EFP>
__device__ __forceinline__ bool n3_column(const KP &p, const PairSys &ps, int J, N3Warp<RF> &w) {
  constexpr unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int ntot = ps.ntot, nt = p.nion_t;
  const int jl = ps.nsites + J * 32 + lane;
  float4 h = make_float4(1e10f, 1e10f, 1e10f, __int_as_float(EFP ? 0 : p.ndna));
  float4 l = make_float4(0.f, 0.f, 0.f, 0.f), u = l;
  if (jl < ntot) {
    h = __ldcg(ps.pk1 + jl);
    l = __ldcg(ps.pk2 + jl);
    if (RF) u = __ldcg(ps.pk3 + jl);
  }
  const int hcode = __float_as_int(h.w);
  const int lcol = EFP ? 0 : (jl < ntot ? (hcode & 0xffff) - p.ndna : nt);
  const float hx = __shfl_xor_sync(kAll, h.x, 16), hy = __shfl_xor_sync(kAll, h.y, 16),
              hz = __shfl_xor_sync(kAll, h.z, 16), lx = __shfl_xor_sync(kAll, l.x, 16),
              ly = __shfl_xor_sync(kAll, l.y, 16), lz = __shfl_xor_sync(kAll, l.z, 16),
              lw = __shfl_xor_sync(kAll, l.w, 16);
  const int lc = __shfl_xor_sync(kAll, lcol, 16);
  w.p0[lane] = make_float4(h.x, hx, h.y, hy);
  w.p1[lane] = make_float4(h.z, hz, l.x, lx);
  w.p2[lane] = make_float4(l.y, ly, l.z, lz);
  w.p3[lane] = make_float4(__int_as_float(lcol), __int_as_float(lc), l.w, lw);
  const int sb0 = __float_as_int(u.z);
  if (RF) {
    const float ux = __shfl_xor_sync(kAll, u.x, 16), uy = __shfl_xor_sync(kAll, u.y, 16);
    w.p4[lane] = make_float4(u.x, ux, u.y, uy);
    w.ab[lane] = make_float2(0.f, 0.f);
    w.cflag[lane] = sb0;
  }
  w.a0[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  w.a1[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
  w.code[lane] = hcode;
  bool ok = jl >= ntot || jl >= ps.nsites + ps.nfix;
  if (RF) ok = ok && (jl >= ntot || (sb0 & 12) == 12 || !(sb0 & 1));
  return ok;
}

// Fast loop of an item's NR row tiles against its column tile (off-diagonal
// tile pairs whose ions are all present and mobile, analytic laws): at step
// k = 0..15 lane l meets column entries m = (l + k) mod 32 and m ^ 16 as the
// two halves of packed f32x2 arithmetic, once per row tile, so one read of a
// column slot and one update of its sums serve 2 NR pairs.  SRPMF pairs are
// queued in (step, row tile, half, lane) order: row lane | column entry << 5
// | row tile << 10.
template <int NR, bool RF, bool PBC>
__device__ __forceinline__ void n3_fast(const KP &p, N3Warp<RF> &w, const float4 *tab,
                                        const N3Row (&r)[NR], N3Sum (&S)[NR], float e[5]) {
  constexpr unsigned kAll = 0xffffffffu;
  constexpr int kStep = 64 * NR;  // SRPMF entries one step can queue
  constexpr int kUnroll = 2;
  const int lane = threadIdx.x & 31;
  float2 THX[NR], THY[NR], THZ[NR], TLX[NR], TLY[NR], TLZ[NR], SRT[NR], RFT[NR], CT[NR];
  const float4 *tr[NR];
#pragma unroll
  for (int a = 0; a < NR; ++a) {
    THX[a] = v2(r[a].th.x);
    THY[a] = v2(r[a].th.y);
    THZ[a] = v2(r[a].th.z);
    TLX[a] = v2(r[a].tl.x);
    TLY[a] = v2(r[a].tl.y);
    TLZ[a] = v2(r[a].tl.z);
    SRT[a] = v2(r[a].srt);
    RFT[a] = v2(r[a].rft);
    CT[a] = v2(r[a].ct);
    tr[a] = tab + r[a].row;
  }
  const unsigned below = (1u << lane) - 1u;
  float2 E0 = v2(0.f), E1 = v2(0.f), E4 = v2(0.f);
  int qn = 0;  // queued SRPMF pairs (warp-uniform)
  auto srp_flush = [&]() {  // warp-uniform
    for (int b = 0; b < qn; b += 32) {
      const int idx = b + lane;
      const bool act = idx < qn;
      const int ent = act ? w.q[idx] : 0;
      const int rl = ent & 31, j = (ent >> 5) & 31, ra = ent >> 10;
      // the row ion's records: lane rl of row tile ra
      float4 rh = make_float4(0.f, 0.f, 0.f, 0.f), rlo = rh;
      int rcode = 0;
#pragma unroll
      for (int a = 0; a < NR; ++a) {
        const float hx = __shfl_sync(kAll, r[a].th.x, rl), hy = __shfl_sync(kAll, r[a].th.y, rl),
                    hz = __shfl_sync(kAll, r[a].th.z, rl), lx = __shfl_sync(kAll, r[a].tl.x, rl),
                    ly = __shfl_sync(kAll, r[a].tl.y, rl), lz = __shfl_sync(kAll, r[a].tl.z, rl);
        const int c = __shfl_sync(kAll, r[a].tcode, rl);
        if (a == ra) {
          rh = make_float4(hx, hy, hz, 0.f);
          rlo = make_float4(lx, ly, lz, 0.f);
          rcode = c;
        }
      }
      float gx = 0.f, gy = 0.f, gz = 0.f;
      if (act) {
        float4 ch, cl;
        n3_entry(w, j, ch, cl);
        // the r^2 of the loop, operation for operation
        float dx = (rh.x - ch.x) + (rlo.x - cl.x);
        float dy = (rh.y - ch.y) + (rlo.y - cl.y);
        float dz = (rh.z - ch.z) + (rlo.z - cl.z);
        if (PBC) min_image_f(p, dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float ds =
            srpmf32(p, srp_index(p, rcode, w.code[j]), r2, rsqrt_nz(r2), 1.0f, e,
                    srp_branch(p, r2, [&] { return pair_r2_64<PBC>(p, rh, rlo, ch, cl); }));
        gx = ds * dx;
        gy = ds * dy;
        gz = ds * dz;
      }
      const int nb = min(32, qn - b);
      for (int t = 0; t < nb; ++t) {  // queue order
        const int rt = __shfl_sync(kAll, rl, t), jt = __shfl_sync(kAll, j, t),
                  at = __shfl_sync(kAll, ra, t);
        const float vx = __shfl_sync(kAll, gx, t), vy = __shfl_sync(kAll, gy, t),
                    vz = __shfl_sync(kAll, gz, t);
        if (lane == rt) {
#pragma unroll
          for (int a = 0; a < NR; ++a)
            if (a == at) {
              S[a].fx.x += vx;
              S[a].fy.x += vy;
              S[a].fz.x += vz;
            }
          float4 c = w.a0[jt];
          c.x += vx;
          c.z += vy;
          w.a0[jt] = c;
          w.a1[jt].x += vz;
        }
        __syncwarp();
      }
    }
    qn = 0;
  };
#pragma unroll(kUnroll)
  for (int k = 0; k < 16; ++k) {
    const int m = (lane + k) & 31;
    const float4 P0 = w.p0[m], P1 = w.p1[m], P2 = w.p2[m], P3 = w.p3[m];
    const float4 A0 = w.a0[m], A1 = w.a1[m];
    float4 P4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 cb = v2(0.f);
    if (RF) {
      P4 = w.p4[m];
      cb = w.ab[m];
    }
    float2 cx = v2(A0.x, A0.y), cy = v2(A0.z, A0.w), cz = v2(A1.x, A1.y), ca = v2(A1.z, A1.w);
    const int col0 = __float_as_int(P3.x), col1 = __float_as_int(P3.y);
#pragma unroll
    for (int a = 0; a < NR; ++a) {
      float2 dx = v2add(v2sub(THX[a], v2(P0.x, P0.y)), v2sub(TLX[a], v2(P1.z, P1.w)));
      float2 dy = v2add(v2sub(THY[a], v2(P0.z, P0.w)), v2sub(TLY[a], v2(P2.x, P2.y)));
      float2 dz = v2add(v2sub(THZ[a], v2(P1.x, P1.y)), v2sub(TLZ[a], v2(P2.z, P2.w)));
      if (PBC) {
        min_image_f(p, dx.x, dy.x, dz.x);
        min_image_f(p, dx.y, dy.y, dz.y);
      }
      const float2 r2 = v2fma(dx, dx, v2fma(dy, dy, v2mul(dz, dz)));
      float4 c0 = tr[a][col0], c1 = tr[a][col1];
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
      const bool s0 = r2.x <= c0.w, s1 = r2.y <= c1.w;
      const unsigned b0 = __ballot_sync(kAll, s0), b1 = __ballot_sync(kAll, s1);
      if (b0 | b1) {
        if (s0) w.q[qn + __popc(b0 & below)] = lane | (m << 5) | (a << 10);
        if (s1) w.q[qn + __popc(b0) + __popc(b1 & below)] = lane | ((m ^ 16) << 5) | (a << 10);
        qn += __popc(b0) + __popc(b1);
      }
      if (RF) {
        const float2 reff = v2(P4.x, P4.y), srfe = v2(P3.z, P3.w);
        const float2 rij = v2mul(reff, RFT[a]), srij = v2mul(srfe, SRT[a]);
        const float2 tt = v2fma(rij, rij, r2);
        const float2 rfdn = v2(rsqrt_nz(tt.x), rsqrt_nz(tt.y));
        const float2 aux0 = v2mul(CT[a], v2(P4.z, P4.w));
        const float2 a1 = v2mul(v2mul(aux0, rij), rfdn);
        E4 = v2fma(a1, srij, E4);
        const float2 a2 = v2mul(v2mul(v2mul(v2mul(aux0, srij), rfdn), rfdn), rfdn);
        const float2 a2p = v2mul(a2, v2fma(rij, v2(0.5f), r2));
        S[a].na = v2fma(a1, srfe, S[a].na);
        S[a].nb = v2fma(a2p, reff, S[a].nb);
        de = v2fma(a2, rij, de);
        ca = v2fma(a1, SRT[a], ca);
        cb = v2fma(a2p, RFT[a], cb);
      }
      S[a].fx = v2fma(de, dx, S[a].fx);
      S[a].fy = v2fma(de, dy, S[a].fy);
      S[a].fz = v2fma(de, dz, S[a].fz);
      cx = v2fma(de, dx, cx);
      cy = v2fma(de, dy, cy);
      cz = v2fma(de, dz, cz);
    }
    w.a0[m] = make_float4(cx.x, cx.y, cy.x, cy.y);
    w.a1[m] = make_float4(cz.x, cz.y, ca.x, ca.y);
    if (RF) w.ab[m] = cb;
    __syncwarp();
    if (qn > kSrpQ - kStep) srp_flush();
  }
  if (qn) srp_flush();
  e[0] += E0.x + E0.y;
  e[1] += E1.x + E1.y;
  e[4] += E4.x + E4.y;
}

// General loop of one row tile against the column tile: any mix of present,
// absent, fixed and mobile ions, tabulated laws, and the diagonal tile pair
// (each pair once: k = 1..16, the last step by the lower half of the lanes).
template <bool II, bool RF, bool EFP, bool PBC>
__device__ __forceinline__ void n3_general(const KP &p, const PairSys &ps, const N3Row &r, int J,
                                           bool diag, int ncol, N3Warp<RF> &w, const float4 *tab,
                                           N3Sum &S, float e[5]) {
  const int lane = threadIdx.x & 31;
  const int m0 = ps.nsites + ps.nfix;
  const int k0 = diag ? 1 : 0, k1 = diag ? 16 : 31;
  for (int k = k0; k <= k1; ++k) {
    const int mm = (lane + k) & 31;
    if (r.iv && mm < ncol && !(diag && k == 16 && lane >= 16)) {
      float4 hc, lc;
      n3_entry(w, mm, hc, lc);
      const int scode = w.code[mm];
      const int j = ps.nsites + J * 32 + mm;
      const bool smob = j >= m0;
      float dx = (r.th.x - hc.x) + (r.tl.x - lc.x);
      float dy = (r.th.y - hc.y) + (r.tl.y - lc.y);
      float dz = (r.th.z - hc.z) + (r.tl.z - lc.z);
      if (PBC) min_image_f(p, dx, dy, dz);
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      auto r2d = [&] { return pair_r2_64<PBC>(p, r.th, r.tl, hc, lc); };
      float dii = 0.0f, drf = 0.0f, dAs = 0.0f, dBs = 0.0f;
      if (II && (r.tmob || smob) && !(PBC && r2 >= p.f.rc2)) {
        if (EFP) {
          dii = law32k(p, __ldg(p.pidx + r.row + (scode & 0xffff)), r2, 1.0f, e, r2d);
        } else {
          const float4 c = tab[r.row + (scode & 0xffff) - p.ndna];
          const float ir = rsqrt_nz(r2), ir2 = ir * ir;
          const float cofo = c.x * ir;
          e[0] += cofo;
          float d6 = c.z * ir2;
          d6 = d6 * d6 * d6;
          const float d12 = d6 * d6;
          e[1] = fmaf(c.y, d12 - d6, e[1]);
          dii = ir2 * fmaf(c.y, fmaf(2.0f, d12, -d6), cofo);
          if (r2 <= c.w)
            dii += srpmf32(p, srp_index(p, r.tcode, scode), r2, ir, 1.0f, e,
                           srp_branch(p, r2, r2d));
        }
      }
      if (RF) {
        const float4 P4 = w.p4[mm];
        const int sb = w.cflag[mm];
        if (r.i > j ? ((r.tb & 4) && (sb & 8)) : ((sb & 4) && (r.tb & 8))) {
          const float rij = P4.x * r.rft, srij = lc.w * r.srt;
          const float rfdn = rsqrt_nz(fmaf(rij, rij, r2));
          const float aux0 = r.ct * P4.z;
          const float a1 = aux0 * rij * rfdn;
          e[4] = fmaf(a1, srij, e[4]);
          const float a2 = aux0 * srij * rfdn * rfdn * rfdn;
          const float a2p = a2 * fmaf(rij, 0.5f, r2);
          S.na.x = fmaf(a1, lc.w, S.na.x);
          S.nb.x = fmaf(a2p, P4.x, S.nb.x);
          dAs = a1 * r.srt;
          dBs = a2p * r.rft;
          drf = a2 * rij;
        }
      }
      const float dt = (r.tmob ? dii : 0.0f) + drf, ds = (smob ? dii : 0.0f) + drf;
      S.fx.x = fmaf(dt, dx, S.fx.x);
      S.fy.x = fmaf(dt, dy, S.fy.x);
      S.fz.x = fmaf(dt, dz, S.fz.x);
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

// Row side of tile pair q: lane l = row ion l.
template <bool RF>
__device__ __forceinline__ void n3_out_row(const PairSys &ps, int q, int qforces, bool iv,
                                           const N3Sum &S) {
  const int lane = threadIdx.x & 31;
  const bool on = qforces && iv;
  ps.tpf[(size_t)q * 64 + lane] =
      on ? make_float4(S.fx.x + S.fx.y, S.fy.x + S.fy.y, S.fz.x + S.fz.y, -(S.na.x + S.na.y))
         : make_float4(0.f, 0.f, 0.f, 0.f);
  if (RF) ps.tpb[(size_t)q * 64 + lane] = on ? -(S.nb.x + S.nb.y) : 0.f;
}

// Column side of tile pair q: lane l = column entry l, the first half of
// slot l plus the second half of slot l ^ 16; zeros where `on` is false.
template <bool RF>
__device__ __forceinline__ void n3_out_col(const PairSys &ps, int q, bool on, const N3Warp<RF> &w) {
  const int lane = threadIdx.x & 31;
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  float b = 0.f;
  if (on) {
    const float4 X0 = w.a0[lane], Y0 = w.a0[lane ^ 16], X1 = w.a1[lane], Y1 = w.a1[lane ^ 16];
    v = make_float4(-(X0.x + Y0.y), -(X0.z + Y0.w), -(X1.x + Y1.y), -(X1.z + Y1.w));
    if (RF) b = -(w.ab[lane].x + w.ab[lane ^ 16].y);
  }
  ps.tpf[(size_t)q * 64 + 32 + lane] = v;
  if (RF) ps.tpb[(size_t)q * 64 + 32 + lane] = b;
}

// Work item `it` of the Newton-3 pair kernels (n3_item, or with one row
// tile per item the tile pair n3_pair), run by one warp
// (all 32 lanes).  w: the warp's shared arrays; tab: the block's dense
// ion-ion law table (rows of ipq_stride(nt)); e: the lane's energy sums
// (ecoul, elj, esrpmf, eefpot, erfpar), added to; without EFP the elj sum
// holds 6 x elj (the dense table holds 6 epp4).  p: the laws and constants.
// An item of two row tiles writes both tile pairs' row sides; the column
// sums of both rows go to the first tile pair's column side and the
// second's is zero.
template <bool II, bool RF, bool EFP, bool PBC = false>
__device__ __forceinline__ void n3_tile(const KP &p, const PairSys &ps, int it, int qforces,
                                        N3Warp<RF> &w, const float4 *tab, float e[5]) {
  constexpr unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int T = ps.T;
  int I, I2 = -1, J;
  if (ps.rows == 2)
    n3_item(T, it, I, I2, J);
  else
    n3_pair(T, it, I, J);
  __syncwarp();  // the warp's arrays may still hold the previous item
  const bool cok = n3_column<RF, EFP>(p, ps, J, w);
  const bool jv = ps.nsites + J * 32 + lane < ps.ntot;
  const int ncol = min(32, max(0, ps.ntot - (ps.nsites + J * 32)));
  N3Row rr[2];
  rr[0] = n3_row<RF, EFP>(p, ps, I);
  if (I2 >= 0) rr[1] = n3_row<RF, EFP>(p, ps, I2);
  __syncwarp();
  N3Sum S[2] = {};
  const int qa = n3_index(T, I, J);
  if (I2 < 0) {
    const bool diag = I == J;
    if (II && !EFP && !diag && __all_sync(kAll, cok && n3_row_fast<RF>(rr[0]))) {
      const N3Row r1[1] = {rr[0]};
      N3Sum s1[1] = {};
      n3_fast<1, RF, PBC>(p, w, tab, r1, s1, e);
      S[0] = s1[0];
    } else {
      n3_general<II, RF, EFP, PBC>(p, ps, rr[0], J, diag, ncol, w, tab, S[0], e);
    }
    n3_out_row<RF>(ps, qa, qforces, rr[0].iv, S[0]);
    n3_out_col<RF>(ps, qa, qforces && jv, w);
    return;
  }
  if (II && !EFP &&
      __all_sync(kAll, cok && n3_row_fast<RF>(rr[0]) && n3_row_fast<RF>(rr[1]))) {
    n3_fast<2, RF, PBC>(p, w, tab, rr, S, e);
  } else {
    n3_general<II, RF, EFP, PBC>(p, ps, rr[0], J, false, ncol, w, tab, S[0], e);
    n3_general<II, RF, EFP, PBC>(p, ps, rr[1], J, false, ncol, w, tab, S[1], e);
  }
  const int qb = n3_index(T, I2, J);
  n3_out_row<RF>(ps, qa, qforces, rr[0].iv, S[0]);
  n3_out_row<RF>(ps, qb, qforces, rr[1].iv, S[1]);
  n3_out_col<RF>(ps, qa, qforces && jv, w);
  n3_out_col<RF>(ps, qb, false, w);
}

}  // namespace bgpu
