// Host-side launch interface between the C ABI (api.cu) and the kernels.
#pragma once
#include "kparams.cuh"

namespace bgpu {

// A pair of CUDA events bracketing one launch (diagnostic timing).
struct KTimer {
  cudaEvent_t a, b;
};

struct EnergyPlan {
  int ntot_ub;        // host upper bound of the device-resident ntot
  int nchunk_ii;      // source chunks of the ion-ion kernel
  int nchunk_rf;      // source chunks of the RFPAR cross kernel
  bool fp32;
  bool reduce_energy; // launch the final energy reduction
  KTimer *t_pairs = nullptr, *t_rf = nullptr, *t_fields = nullptr;
};

struct AssembleFlags {
  int ii, is, rf;     // which partial-force buffers are valid
  int nchunk_ii, nchunk_rf;
  int fp32_noise;     // single-precision Box-Muller (FP32 mode)
};

// fields.cu: single-particle terms, one warp per particle
int fields_blocks(int ntot_ub);
void launch_fields(const KP &p, int ntot_ub, uint32_t mask, int qforces, bool fp32,
                   int slot0, cudaStream_t stream);

// energy.cu
int launch_energy(const KP &p, const EnergyPlan &plan, uint32_t mask,
                  int qforces, cudaStream_t stream);
int energy_slots(const KP &p, const EnergyPlan &plan, uint32_t mask);

// dyn.cu: force assembly, optionally fused with the BD update
void launch_assemble(const KP &p, int ntot_ub, const AssembleFlags &fl,
                     int do_bd, int variant, uint64_t seed, uint64_t step,
                     cudaStream_t stream);

// gcmc.cu
void launch_interact(const KP &p, int ntot_ub, uint32_t mask, int qalert,
                     double *dener_dev, cudaStream_t stream);
void launch_gcmc_attempt(const KP &p, int ntot_ub, uint32_t mask,
                         uint64_t seed, uint64_t cycle, uint32_t attempt,
                         cudaStream_t stream);
int interact_slots(int ntot_ub);

}  // namespace bgpu

// Read-only view of a context's uploaded pair laws, for entry points that
// live outside api.cu.  Returns false until set_system/types/pairs are done.
struct bromoc_ctx;
bool bromoc_ctx_pair_view(const bromoc_ctx *ctx, const bgpu::KP **kp,
                          cudaStream_t *stream, int *precision);
int bromoc_ctx_fail(bromoc_ctx *ctx, int code, const char *msg);
