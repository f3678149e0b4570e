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
  int ntile;          // FP32: ion tiles of the Newton-3 pair kernel (0: chunked)
  bool fp32;
  bool cells = false; // FP32 extension mode: the cell-list pair kernel
  bool reduce_energy; // launch the final energy reduction
  bool nuc = false;   // DNA bonded/Go terms (nucl.cu)
  bool mmij = false;  // MMIJ reaction field (mmij.cu)
  KTimer *t_pairs = nullptr, *t_rf = nullptr, *t_fields = nullptr;
};

// Tile pairs (I <= J) of the Newton-3 pair kernel, row-major: row I holds
// J = I..T-1 and starts at offset I T - I (I - 1) / 2.
constexpr int kN3MaxTiles = 256;  // up to 8192 ions; beyond, the chunked kernel
// Sites per tile of the FP32 ion-site pair kernel: a warp's 32 ions meet
// them one after another.
constexpr int kIsSiteTile = 8;
__host__ __device__ inline int n3_pairs(int T) { return T * (T + 1) / 2; }
__host__ __device__ inline int n3_index(int T, int I, int J) {
  return I * T - I * (I - 1) / 2 + (J - I);
}
// Work items of the Newton-3 pair kernels, column tile by column tile:
// column J's off-diagonal row tiles 0..J-1 go in pairs (2s, 2s+1), one item
// of 64 row ions against the column's 32 entries; when J is odd, row tile
// J-1 is an item of its own; the diagonal tile pair (J, J) comes last.
// Items before column J: J + floor(J^2 / 4).
__host__ __device__ inline int n3_items_before(int J) { return J + J * J / 4; }
__host__ __device__ inline int n3_items(int T) { return n3_items_before(T); }
// Tile pair q of the row-major list: (I, J).
__host__ __device__ inline void n3_pair(int T, int q, int &I, int &J) {
  const float b = 2.0f * T + 1.0f;
  int i = (int)((b - sqrtf(b * b - 8.0f * q)) * 0.5f);
  i = i < 0 ? 0 : (i > T - 1 ? T - 1 : i);
  while (i > 0 && n3_index(T, i, i) > q) --i;
  while (i + 1 < T && n3_index(T, i + 1, i + 1) <= q) ++i;
  I = i;
  J = i + (q - n3_index(T, i, i));
}
// Item it of T tiles: column J and row tiles I, I2 (I2 < 0: one row tile).
__host__ __device__ inline void n3_item(int T, int it, int &I, int &I2, int &J) {
  int j = (int)(2.0f * (sqrtf((float)it + 1.0f) - 1.0f));
  j = j < 0 ? 0 : (j > T - 1 ? T - 1 : j);
  while (j > 0 && n3_items_before(j) > it) --j;
  while (j + 1 < T && n3_items_before(j + 1) <= it) ++j;
  const int s = it - n3_items_before(j), nd = j >> 1;
  J = j;
  I2 = -1;
  if (s < nd) {
    I = 2 * s;
    I2 = 2 * s + 1;
  } else {
    I = (j & 1) && s == nd ? j - 1 : j;
  }
}

// Targets of the FP32 pair kernel: ion-ion terms act on mobile ions, the
// RFPAR cross term on every ion in the map, so with RFPAR on the targets
// start at the first ion, else at the first mobile ion.
struct PairCfg32 {
  bool ii, rf;
  int t0, ntg;  // first target, number of target slots below ntot_ub
};
inline PairCfg32 pair_cfg32(const KP &p, int ntot_ub, uint32_t mask) {
  PairCfg32 c{};
  c.ii = (mask & 1u) && ntot_ub > p.nsites + p.nfix;
  c.rf = (mask & 16u) && p.qrfpar && ntot_ub > p.nsites;
  c.t0 = c.rf ? p.nsites : p.nsites + p.nfix;
  c.ntg = (c.ii || c.rf) ? ntot_ub - c.t0 : 0;
  return c;
}

struct AssembleFlags {
  int ii, is, rf;     // which partial-force buffers are valid
  int ii_from;        // first particle with ion-ion (fused FP32: pair) partials
  int nchunk_ii, nchunk_rf;
  int fp32_noise;     // single-precision Box-Muller (FP32 mode)
  int fp32_partials;  // FP32 mode: float partials, float-float positions
  int use_total;      // the force is fx,fy,fz as assembled earlier (dynamics())
  int ntile;          // FP32: partials are per tile pair (Newton-3 kernel)
  int rf_ab;          // FP32 Newton-3: add A sd1 + B sd2 of the RFPAR chain
};

// mmij.cu: MMIJ reaction field (energy into slot `slot`, forces added to
// ffield / ffield_f); INTERACT's term of p.trial added to *dener
int mmij_chunks(const KP &p, int ntot_ub);
int mmij_table_width(int rect, int nx, int ny, int nz, int nmpol);
int launch_mmij(const KP &p, bool fp32, int ntot_ub, int qforces, int slot,
                cudaStream_t stream);
void launch_mmij_interact(const KP &p, int ntot_ub, double *dener, cudaStream_t stream);

// gcmc.cu: COUNT (count.f90) on the device; ff: positions from the
// float-float records
int launch_count(const KP &p, bool ff, int ntot_ub, cudaStream_t stream);  // launches

// analysis.cu: per-cycle profiles (counts) and .btr frames
struct ProfArgs {
  int rho, rdna, gr;        // which profiles accumulate
  double zmini, idelz;      // z bins: iz = int((z - zmini) idelz) + 1
  int nzmax;
  int igr, npoints;         // RDF centre (0-based) and shells
  double dr;
  unsigned long long *rho_n, *rdna_n, *gr_n;  // [(ntype-nold)*nzmax], [ndna*nzmax], [(ntype-nold)*npoints]
  int *irmax;
};
void launch_profiles(const KP &p, bool fp32, int ntot_ub, const ProfArgs &a,
                     cudaStream_t stream);
void launch_traj_pack(const KP &p, bool fp32, int n, double runtime, uint32_t *w,
                      cudaStream_t stream);

// nucl.cu: DNA bonded and Go-like terms; forces into fis / fis_f of the
// sites (added when accum, else written), energies into one slot
int launch_nucl(const KP &p, bool fp32, uint32_t mask, int qforces, int accum, int slot,
                cudaStream_t stream);
int nucl_slots(const KP &p);  // energy slots launch_nucl writes
// NOTRAN after a BD step: the sites' centre back to notr along the flagged
// axes (one block); returns the launches (0 when off)
int launch_notrans(const KP &p, bool fp32, cudaStream_t stream);
// INTERACT of site j (0-based): adds its bonded/Go terms to *dener
void launch_nucl_interact(const KP &p, uint32_t mask, int j, double *dener,
                          cudaStream_t stream);

// fields.cu: single-particle terms, one warp per particle
int fields_blocks(int ntot_ub);
void launch_fields(const KP &p, int ntot_ub, uint32_t mask, int qforces, bool fp32,
                   int slot0, cudaStream_t stream);
// FP32 mode: FP64 coordinates -> float-float records (to_records) or back
void launch_pack(const KP &p, int ntot_ub, bool to_records, cudaStream_t stream);

// energy.cu
int launch_energy(const KP &p, const EnergyPlan &plan, uint32_t mask,
                  int qforces, cudaStream_t stream);
int energy_slots(const KP &p, const EnergyPlan &plan, uint32_t mask);
// cells.cu: the cell list of the FP32 extension mode and its pair kernel
// (block partial energies from `slot`); returns the kernels launched
int launch_cells(const KP &p, int ntot_ub, int qforces, int slot, cudaStream_t stream);
int cell_pair_blocks(const KP &p, int ntot_ub);
// Row tiles per work item of the Newton-3 pair kernels for T tiles: two
// (n3_item) when the tile pairs outnumber one wave of warps (16 a SM), so a
// column read serves more pairs; else one (each tile pair an item, the
// row-major list), for the shorter chain per warp.
int n3_rows(int T);
__host__ __device__ inline int n3_work(int T, int rows) { return rows == 2 ? n3_items(T) : n3_pairs(T); }
int n3_blocks(int ntile);  // blocks (energy slots) of the Newton-3 pair kernel

// dyn.cu: force assembly, optionally fused with the BD update
void launch_assemble(const KP &p, int ntot_ub, const AssembleFlags &fl,
                     int do_bd, int variant, uint64_t seed, uint64_t step,
                     cudaStream_t stream);

// loop.cu: nsteps fused BD steps of the FP32 Newton-3 path in one
// cooperative launch (fields_first: evaluate the single-particle terms first)
bool bd_loop_supported(const KP &p, const AssembleFlags &fl);
cudaError_t launch_bd_loop(const KP &p, const AssembleFlags &fl, int ntot_ub, uint32_t mask,
                           int variant, uint64_t seed, uint64_t step0, int nsteps,
                           int fields_first, cudaStream_t stream);

// gcmc.cu
// Metropolis moves (mc.cu): the chain's device record, reset per call.
struct McState {
  int iat, skip, draw, naccept;  // the move's ion (0-based), no position found, next draw
  double xn, yn, zn;             // its proposed position
  double e[2];                   // INTERACT at the old and the new position
  double dener;                  // accepted energy change of the call
};
int launch_metropolis(const KP &p, int ntot, uint32_t mask, int nmcm, double mcmax,
                      uint64_t seed, uint64_t cycle, McState *mc, cudaStream_t stream);

void launch_interact(const KP &p, int ntot_ub, uint32_t mask, int qalert,
                     double *dener_dev, cudaStream_t stream);
// gcmc.cu: GRAND one attempt after another (systems with the MMIJ reaction
// field): proposal, INTERACT into *de_dev, acceptance, per attempt; the
// FP64 arrays move; returns the launches
int launch_grand_seq(const KP &p, int ntot_ub, uint32_t mask, uint64_t seed, uint64_t cycle,
                     int ngcmc, double *de_dev, cudaStream_t stream);
// GRAND: ngcmc attempts in one cooperative launch (gcmc.cu)
// ffpos: FP32 mode, positions in the float-float records (pk1, pk2)
cudaError_t launch_grand(const KP &p, int ntot_ub, int ipart_slots, uint32_t mask,
                         uint64_t seed, uint64_t cycle, int ngcmc, int ffpos,
                         cudaStream_t stream);
// partial slots for GRAND's widest grid at capacity cap (a lane per
// particle and attempt); INTERACT's need at cap is smaller
int grand_slots(int cap);
int interact_slots(int ntot_ub);

}  // namespace bgpu

// Read-only view of a context's uploaded pair laws, for entry points that
// live outside api.cu.  Returns false until set_system/types/pairs are done.
struct bromoc_ctx;
bool bromoc_ctx_pair_view(const bromoc_ctx *ctx, const bgpu::KP **kp,
                          cudaStream_t *stream, int *precision);
int bromoc_ctx_fail(bromoc_ctx *ctx, int code, const char *msg);
// FP32 prototype for a replica batch: completes its setup (scratch, FP32
// constants) and returns its parameter block.
int bromoc_ctx_prepare_f32(bromoc_ctx *ctx, const bgpu::KP **kp, cudaStream_t *stream);
// Replica batches and adjoint engines borrow their prototype context's
// stream and tables.  They attach a flag to it; a context destroyed before
// them sets the flag, and they then neither touch its stream nor run.
void bromoc_ctx_attach(bromoc_ctx *ctx, int *orphaned);
void bromoc_ctx_detach(bromoc_ctx *ctx, int *orphaned);
