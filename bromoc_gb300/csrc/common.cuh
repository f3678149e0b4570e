// Shared device-side definitions of the GB300 cg-gcmc-bd inner loop.
//
// Layout in HBM (one context):
//   particles  SoA double x,y,z [cap], int typei,ibuffer [cap]; sites first,
//              then fixed ions, then mobile ions (energy.mono.f90:120-123)
//   forces     double fx,fy,fz [cap] (assembled), partial-force scratch
//   pair laws  PairParam[ntc] + pair index table [nttyp*nttyp] (nindex.f90)
//   tables     ep double[3*cnt] (reference form) and a float4 local form
//   maps       phix float, phiv int8, gsrfen/greff float; z fastest
//   live state DevState {ntot, nat[], counters, error flag}: device-resident
//              so that GCMC insertions/deletions need no host round trip.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bgpu {

constexpr double kPi = 3.14159265358979323846264338327950288419716939937510;
constexpr double kTwoPi = 2.0 * kPi;
constexpr double kRsmall = 1E-3;  // constamod.f90:83
constexpr int kNTerms = 23;       // BROMOC_NTERMS
constexpr int kMaxBuffers = 64;
constexpr int kMaxTypes = 64;
constexpr int kIonTabTypes = 16;  // ion types of the shared-memory pair table
// Row stride of that table: each row of ion type a holds its nt laws (a, b)
// and, at column nt, a zero law that empty column slots of a pair tile use.
__host__ __device__ constexpr int ipq_stride(int nt) { return nt + 1; }
constexpr int kIpqMax = kIonTabTypes * (kIonTabTypes + 1);

// ---- packed FP32 pairs (f32x2, sm_100 and later) ---------------------------
// One instruction applies the operation to both halves; each half rounds as
// the scalar operation would.
__device__ __forceinline__ float2 v2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 v2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 v2fma(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2 v2sub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 v2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 v2(float a) { return make_float2(a, a); }

// Hint to bring the line holding *a into L2 (no result; a lies inside an
// allocation).
__device__ __forceinline__ void prefetch_l2(const void *a) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

// error flags raised by kernels (bit mask in DevState::err)
enum : int {
  kErrCapacity = 1,     // an insertion would exceed capacity
  kErrTableIndex = 2,   // an effective-potential piece index out of range
  kErrFind = 4,         // GCMC deletion could not find the particle
  kErrBounds = 8,       // a guarded index was out of range (access skipped)
  kErrBarrier = 16,     // a grid barrier gave up waiting (the kernel returned)
  kErrOutside = 32,     // COUNT found a buffer ion outside the system
};

// packed pair-law switches
enum : int { kChr = 1, kLj = 2, kSrp = 4, kEfp = 8 };

struct PairParam {
  double fct, epp4, sgp2;
  double c0, c1, c2, c3, c4;
  double sc0, sc1, sc2;     // core a/r^12 + b, tail a/r^6
  double dm2lo, dm2hi, dmi;
  int flags;
  int nxi;                  // 0-based first piece
  int npieces;
  int pad;
};

// Device-resident live counters of one context.
struct DevState {
  int ntot;
  int err;
  int bad_site, bad_index, bad_bound, pad_;  // first guarded violation
  int nat[kMaxBuffers];
  int ninsert[kMaxBuffers];
  int nremove[kMaxBuffers];
  int ntotat[kMaxBuffers];
  double dener_sum;         // accumulated GCMC energy change
  unsigned bar_count;       // grid barriers of the cooperative kernels: arrivals,
  unsigned bar_gen;         // a generation flag and the blocks that have
  unsigned bar_exit;        // finished; all zero between launches (the last
                            // block out of a launch clears them)
  int count_acc[kMaxBuffers];  // COUNT: the blocks' nat sums and the blocks
  unsigned count_done;         // done; zero between launches (the last block
                               // publishes nat and clears them)
};

// GCMC trial of one attempt (written by the proposal kernel).
struct Trial {
  int valid;                // 0: attempt rejected before INTERACT
  int insert;               // 1 insertion, 0 deletion
  int ib;                   // 1-based buffer
  int itype;                // ion type
  int j;                    // 1-based slot (ntot+1 on insertion)
  int draw;                 // next uniform draw index of the attempt
  double x, y, z;
  // single-particle part of INTERACT, filled by one warp before the pair
  // sum: membrane + RFPAR self + static field + repulsion
  double e_single;
  double srfe, reff;        // RFPAR gathers of the trial (0 outside the map)
  int rf_in;                // trial inside the RFPAR map
  int ntot;                 // live particle count when the trial was made
  int chg;                  // GRAND: slot the previous accepted move rewrote, -1 none
};

// GRAND attempts evaluated together in one round of the GRAND kernel.
constexpr int kSpec = 8;

// Header of one GRAND round, written by the coordinating block before it
// publishes the round's trials (Trial[kSpec]).
struct GrandRound {
  int a0, na;               // first attempt of the round, attempts (0: the launch ends)
  int ntot;                 // live particle count the trials were made against
  int nchg;                 // slots the previous round rewrote
  int chg[kSpec];
};

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------
__host__ __device__ inline void philox4x32_10(uint32_t c0, uint32_t c1,
                                              uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1,
                                              uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    uint64_t a = (uint64_t)0xD2511F53u * c0, b = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(a >> 32), lo0 = (uint32_t)a;
    uint32_t hi1 = (uint32_t)(b >> 32), lo1 = (uint32_t)b;
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

__host__ __device__ inline double u01(uint32_t w) { return (double)w * 0x1p-32; }

// Box-Muller, cosine branch (rgauss.f90:24): uniform a -> angle,
// 1 - uniform b -> radius.
__device__ inline double box_muller(uint32_t wa, uint32_t wb) {
  return cos(u01(wa) * kTwoPi) * sqrt(-2.0 * log(1.0 - u01(wb)));
}

// BD noise: 3 Gaussians of particle slot `slot` at step `step`.
__device__ inline void bd_noise3(uint64_t seed, uint64_t step, uint32_t slot,
                                 double g[3]) {
  uint32_t w[4];
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const uint32_t s2 = (uint32_t)step,
                 s3 = ((uint32_t)(step >> 32) & 0x00FFFFFFu) | (1u << 24);
  philox4x32_10(slot, 0u, s2, s3, k0, k1, w);
  g[0] = box_muller(w[0], w[1]);
  g[1] = box_muller(w[2], w[3]);
  philox4x32_10(slot, 1u, s2, s3, k0, k1, w);
  g[2] = box_muller(w[0], w[1]);
}

// Single-precision Box-Muller on the same Philox words: the radius uses
// 1 - u formed exactly in integers (2^32 - w, never 0), the angle
// cos(2 pi u) = cospi(2u).  Differs from the FP64 form by ~1e-7 relative.
__device__ inline float box_muller_f(uint32_t wa, uint32_t wb) {
  const float ua = (float)wa * 0x1p-32f;
  const float u2 = wb == 0u ? 1.0f : (float)(0u - wb) * 0x1p-32f;
  return cospif(2.0f * ua) * sqrtf(-2.0f * logf(u2));
}

__device__ inline void bd_noise3_f(uint64_t seed, uint64_t step, uint32_t slot,
                                   float g[3]) {
  uint32_t w[4];
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const uint32_t s2 = (uint32_t)step,
                 s3 = ((uint32_t)(step >> 32) & 0x00FFFFFFu) | (1u << 24);
  philox4x32_10(slot, 0u, s2, s3, k0, k1, w);
  g[0] = box_muller_f(w[0], w[1]);
  g[1] = box_muller_f(w[2], w[3]);
  philox4x32_10(slot, 1u, s2, s3, k0, k1, w);
  g[2] = box_muller_f(w[0], w[1]);
}

// GCMC uniform draw `draw` of attempt `attempt` of cycle `cycle`.
// The 32-bit word behind gcmc_uniform (the uniform is word * 2^-32).
__host__ __device__ inline uint32_t gcmc_word(uint64_t seed, uint64_t cycle, uint32_t attempt,
                                              uint32_t draw) {
  uint32_t w[4];
  philox4x32_10(attempt, draw >> 2, (uint32_t)cycle,
                ((uint32_t)(cycle >> 32) & 0x00FFFFFFu) | (2u << 24),
                (uint32_t)seed, (uint32_t)(seed >> 32), w);
  return w[draw & 3];
}

__host__ __device__ inline double gcmc_uniform(uint64_t seed, uint64_t cycle,
                                               uint32_t attempt, uint32_t draw) {
  return u01(gcmc_word(seed, cycle, attempt, draw));
}

// The uniforms of Metropolis moves: the GCMC stream's layout under its own
// tag (3), so the two streams never share a counter.
__host__ __device__ inline double mc_uniform(uint64_t seed, uint64_t cycle, uint32_t move,
                                             uint32_t draw) {
  uint32_t w[4];
  philox4x32_10(move, draw >> 2, (uint32_t)cycle,
                ((uint32_t)(cycle >> 32) & 0x00FFFFFFu) | (3u << 24), (uint32_t)seed,
                (uint32_t)(seed >> 32), w);
  return u01(w[draw & 3]);
}

__host__ __device__ inline double fsign(double a, double b) {
  return b >= 0.0 ? fabs(a) : -fabs(a);
}

}  // namespace bgpu
