// Fused BD loop of the FP32 Newton-3 path: nsteps Brownian-dynamics steps
// (dynamics0-3.mono.f90 driven by the ENERGY force of energy.mono.f90) in one
// cooperative launch.  Per step, two phases separated by grid barriers:
//
//   P  every tile pair of ions (the Newton-3 pair tile, one warp each, spread
//      round-robin over the blocks) -> per-tile-pair partial forces;
//   A  one block per half tile of 16 ions (whole tiles of 32 when the half
//      tiles outnumber the blocks): sum the tile's partials in fixed order,
//      add the single-particle forces, move the ions, then evaluate the
//      single-particle terms (maps, RFPAR gathers) at the new positions,
//      one warp per ion, which the next step's phase P reads.
//
// The force terms, their summation order and the noise are those of the
// per-kernel step (fields, pair kernel, assembly), so the positions after a
// call agree with the per-kernel path's.  Energies are not formed here; a
// step whose energy is wanted runs per kernel.  Every barrier wait is
// bounded (gridsync.cuh): a stalled launch records kErrBarrier and returns.
#include <algorithm>

#include "fields32.cuh"
#include "gridsync.cuh"
#include "launch.h"
#include "move32.cuh"
#include "pairs_n3.cuh"

namespace bgpu {

constexpr int kLoopWarps = 16;

// Phase P's per-warp column arrays and phase A's partial sums share the
// block's shared memory (the phases never overlap within a block).
template <bool RF>
union LoopSmem {
  N3Warp<RF> nw[kLoopWarps];
  float part[kLoopWarps][10][32];
};

template <bool II, bool RF, bool EFP, bool PBC>
__global__ void __launch_bounds__(32 * kLoopWarps, 1)
    k_bd_loop(const __grid_constant__ KP p, AssembleFlags fl, uint32_t mask, int variant,
              uint64_t seed, uint64_t step0, int nsteps, int fields_first, int rows) {
  extern __shared__ __align__(16) unsigned char loop_dsm[];  // sizeof(LoopSmem<RF>)
  LoopSmem<RF> &sm = *reinterpret_cast<LoopSmem<RF> *>(loop_dsm);
  __shared__ float4 tab[EFP ? 1 : kIpqMax];
  __shared__ int flag;
  __shared__ AxisF ax[12];
  __shared__ float4 npos[32][3];  // phase A: the moved records of the tile
  stage_axes(p, ax);
  const int nt = p.nion_t;
  if (II && !EFP)
    for (int k = threadIdx.x; k < nt * ipq_stride(nt); k += blockDim.x) tab[k] = __ldg(p.ipq + k);
  __syncthreads();
  const int w = threadIdx.x >> 5;
  const int G = gridDim.x;
  // work slot of this warp: consecutive work items go to consecutive blocks
  const int slot = w * G + blockIdx.x, nslot = G * kLoopWarps;
  const int ntot = p.st->ntot;  // constant during BD
  const int T = fl.ntile, nwork = n3_work(T, rows);
  const PairSys ps = pair_sys(p, ntot, T, rows);
  const AsmSys as = ctx_asm_sys(p, T, seed);
  const int m0 = p.nsites + p.nfix;
  unsigned bar = 0;
  float eo[4];  // single-particle energies: not formed here
  // phase A in half tiles (16 ions a block, one field evaluation a warp)
  // while they fit the grid once, else whole tiles
  const bool halves = 2 * T <= G;
  const int nitem = halves ? 2 * T : T;
  if (fields_first) {
    for (int i = p.nsites + slot; i < ntot; i += nslot)
      fields_one_f32(p, i, false, i < m0, mask, 1, eo, ax);
    if (!grid_barrier(&p.st->bar_count, ++bar, p.st, &flag)) goto done;
  }
  for (int s = 0; s < nsteps; ++s) {
    float e[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int it = slot; it < nwork; it += nslot)
      n3_tile<II, RF, EFP, PBC>(p, ps, it, 1, sm.nw[w], tab, e);
    if (!grid_barrier(&p.st->bar_count, ++bar, p.st, &flag)) goto done;
    for (int it = blockIdx.x; it < nitem; it += G) {
      const int t = halves ? it >> 1 : it, h = halves ? it & 1 : -1;
      assemble_tile<kLoopWarps>(p, as, fl, 1, variant, step0 + s, t, 0, sm.part, h, npos);
      __syncthreads();  // the new positions; part free again
      if (s + 1 < nsteps) {
        const int u0 = halves ? 16 * h : 0;
        for (int u = u0 + w; u < u0 + (halves ? 16 : 32); u += kLoopWarps) {
          const int i = p.nsites + 32 * t + u;
          if (i < ntot) fields_one_f32(p, i, false, i < m0, mask, 1, eo, ax, npos[u]);
        }
      }
    }
    if (s + 1 < nsteps && !grid_barrier(&p.st->bar_count, ++bar, p.st, &flag)) goto done;
  }
done:
  launch_exit(p.st);
}

template <bool II, bool RF, bool EFP, bool PBC = false>
static cudaError_t launch_loop_t(const KP &p, const AssembleFlags &fl, uint32_t mask,
                                 int variant, uint64_t seed, uint64_t step0, int nsteps,
                                 int fields_first, cudaStream_t stream) {
  static int max_res[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  auto kern = k_bd_loop<II, RF, EFP, PBC>;
  const size_t dsm = sizeof(LoopSmem<RF>);
  if (max_res[dev] == 0) {
    int per_sm = 0, nsm = 0;
    if ((e = cudaFuncSetAttribute((const void *)kern,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm)) !=
        cudaSuccess)
      return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kLoopWarps, dsm)) !=
        cudaSuccess)
      return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
      return e;
    // one block per SM at most: every block must be resident at once
    max_res[dev] = per_sm > 0 ? nsm : -1;
  }
  if (max_res[dev] < 0) return cudaErrorCooperativeLaunchTooLarge;
  const int T = fl.ntile;
  const int grid = std::max(1, std::min(max_res[dev], std::max(n3_pairs(T), T)));
  KP pc = p;  // the barrier counters are zero between launches (launch_exit)
  AssembleFlags fc = fl;
  int rows = n3_rows(T);  // as the per-kernel steps' pair launch
  void *args[] = {(void *)&pc,    (void *)&fc,     (void *)&mask,         (void *)&variant,
                  (void *)&seed,  (void *)&step0,  (void *)&nsteps,       (void *)&fields_first,
                  (void *)&rows};
  return cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(32 * kLoopWarps), args,
                                     dsm, stream);
}

bool bd_loop_supported(const KP &p, const AssembleFlags &fl) {
  return fl.fp32_partials && fl.ntile > 0 && !fl.use_total && p.nsites == 0 && !fl.is;
}

cudaError_t launch_bd_loop(const KP &p, const AssembleFlags &fl, int ntot_ub, uint32_t mask,
                           int variant, uint64_t seed, uint64_t step0, int nsteps,
                           int fields_first, cudaStream_t stream) {
  const PairCfg32 pc = pair_cfg32(p, ntot_ub, mask);
  const bool efp = !p.ipq_ok;
  if (p.periodic)  // extension mode: ion-ion only (no RFPAR)
    return efp ? launch_loop_t<true, false, true, true>(p, fl, mask, variant, seed, step0,
                                                        nsteps, fields_first, stream)
               : launch_loop_t<true, false, false, true>(p, fl, mask, variant, seed, step0,
                                                         nsteps, fields_first, stream);
  if (pc.ii && pc.rf)
    return efp ? launch_loop_t<true, true, true>(p, fl, mask, variant, seed, step0, nsteps,
                                                 fields_first, stream)
               : launch_loop_t<true, true, false>(p, fl, mask, variant, seed, step0, nsteps,
                                                  fields_first, stream);
  if (pc.ii)
    return efp ? launch_loop_t<true, false, true>(p, fl, mask, variant, seed, step0, nsteps,
                                                  fields_first, stream)
               : launch_loop_t<true, false, false>(p, fl, mask, variant, seed, step0, nsteps,
                                                   fields_first, stream);
  return launch_loop_t<false, true, true>(p, fl, mask, variant, seed, step0, nsteps,
                                          fields_first, stream);
}

}  // namespace bgpu
