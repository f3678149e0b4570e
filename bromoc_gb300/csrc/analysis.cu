// Per-cycle analysis and trajectory frames on the device.
//
//   k_profiles   simul1.f90:476-509: the z-density profile of the mobile ions
//                (Qrho) and of the DNA sites (Qrdna) in 0.5 A bins from the
//                system's lower z face, and the radial distribution of the
//                mobile ions around particle igr (Qgr), as integer counts
//                (atomic adds of 1 commute, so a run repeats exactly; the
//                reference's real-valued sums of 1.0 are these counts).
//   k_traj_pack  one .btr frame (wrttraj.f90:33-38) as the bytes of six
//                Fortran unformatted sequential records, each framed by
//                4-byte length markers: runtime (real*8), ntot, typtyp(1:ntot)
//                (combined types; ions through nwtype), sng(x), sng(y), sng(z).
#include <algorithm>

#include "launch.h"

namespace bgpu {

constexpr int kAnaThreads = 256;

template <bool F32>
__device__ __forceinline__ void pos3(const KP &p, int i, double r[3]) {
  if (F32) {
    const float4 h = p.pk1[i], l = p.pk2[i];
    r[0] = (double)h.x + (double)l.x;
    r[1] = (double)h.y + (double)l.y;
    r[2] = (double)h.z + (double)l.z;
  } else {
    r[0] = p.x[i];
    r[1] = p.y[i];
    r[2] = p.z[i];
  }
}

template <bool F32>
__global__ void __launch_bounds__(kAnaThreads) k_profiles(KP p, ProfArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntot = p.st->ntot;
  if (i >= ntot) return;
  double r[3];
  pos3<F32>(p, i, r);
  const bool mobile = i >= p.nsites + p.nfix;
  // iz = int((z - zmini) * idelz) + 1, Fortran int() truncating toward zero;
  // bins below 1 (a particle under zmini) are skipped
  const int iz = (int)((r[2] - a.zmini) * a.idelz) + 1;
  if (mobile && a.rho && iz >= 1 && iz <= a.nzmax) {
    const int itype = abs(p.typei[i]) - p.nold;  // 1..ntype-nold
    atomicAdd(a.rho_n + (size_t)(itype - 1) * a.nzmax + (iz - 1), 1ull);
  }
  if (i < p.nsites && a.rdna && iz >= 1 && iz <= a.nzmax)
    atomicAdd(a.rdna_n + (size_t)(p.typtyp[i] - 1) * a.nzmax + (iz - 1), 1ull);
  if (mobile && a.gr && a.igr < ntot) {
    double c[3];
    pos3<F32>(p, a.igr, c);
    const double d2 = (r[0] - c[0]) * (r[0] - c[0]) + (r[1] - c[1]) * (r[1] - c[1]) +
                      (r[2] - c[2]) * (r[2] - c[2]);
    const int ir = (int)(sqrt(d2) / a.dr) + 1;
    atomicMax(a.irmax, min(ir, a.npoints));
    if (ir <= a.npoints) {
      const int itype = abs(p.typei[i]) - p.nold;
      atomicAdd(a.gr_n + (size_t)(itype - 1) * a.npoints + (ir - 1), 1ull);
    }
  }
}

void launch_profiles(const KP &p, bool fp32, int ntot_ub, const ProfArgs &a,
                     cudaStream_t stream) {
  if (ntot_ub <= 0) return;
  const int nb = (ntot_ub + kAnaThreads - 1) / kAnaThreads;
  (fp32 ? k_profiles<true> : k_profiles<false>)<<<nb, kAnaThreads, 0, stream>>>(p, a);
}

// Frame bytes (4-byte words): record k starts with its payload length L_k,
// then the payload, then L_k again.
__host__ __device__ inline long long traj_frame_bytes(int n) {
  return (8 + 8) + (8 + 4) + 4 * (8 + 4 * (long long)n);
}

template <bool F32>
__global__ void __launch_bounds__(kAnaThreads)
    k_traj_pack(KP p, uint32_t *w, int n, double runtime) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t L = 4u * (uint32_t)n;
  // word offsets: runtime record 0..3, ntot record 4..6, then four arrays of
  // n words, each at 7 + k (n + 2) + 1
  if (i == 0) {
    const unsigned long long rb = (unsigned long long)__double_as_longlong(runtime);
    w[0] = 8u;
    w[1] = (uint32_t)rb;  // little-endian real*8
    w[2] = (uint32_t)(rb >> 32);
    w[3] = 8u;
    w[4] = 4u;
    w[5] = (uint32_t)n;
    w[6] = 4u;
    for (int k = 0; k < 4; ++k) {
      w[7 + (size_t)k * (n + 2)] = L;
      w[7 + (size_t)k * (n + 2) + n + 1] = L;
    }
  }
  if (i >= n) return;
  const int t = i < p.nsites ? p.typtyp[i] : p.nwtype[abs(p.typei[i])];
  double r[3];
  pos3<F32>(p, i, r);
  w[8 + i] = (uint32_t)t;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    w[8 + (size_t)(k + 1) * (n + 2) + i] = __float_as_uint(__double2float_rn(r[k]));
}

void launch_traj_pack(const KP &p, bool fp32, int n, double runtime, uint32_t *w,
                      cudaStream_t stream) {
  const int nb = (std::max(n, 1) + kAnaThreads - 1) / kAnaThreads;
  (fp32 ? k_traj_pack<true> : k_traj_pack<false>)<<<nb, kAnaThreads, 0, stream>>>(
      p, w, n, runtime);
}

}  // namespace bgpu
