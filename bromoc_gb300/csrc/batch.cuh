// Replica batches: independent systems that share the prototype context's
// types, pair tables and grid maps, each with its own box, particles and
// noise seed, advanced together by one launch per kernel per BD step.
#pragma once
#include "kparams.cuh"

namespace bgpu {

// One replica on the device.  Its particles occupy slots [off, off + cap)
// of the batch arrays (off a multiple of 32), the first n of them live.
struct RepDev {
  int off, n, cap;
  int w0, w1;      // its pair-tile work items [w0, w1) in the work list
  int rows;        // row tiles per item (n3_rows of its tiles, as a single context)
  int poff;        // its first tile pair in the partial buffers (capacity-sized)
  uint64_t seed;   // BD noise key of this replica
  BoxF box;        // fixcoor constants
};

// GCMC of one replica (grand.f90 on its slots): its buffers, live count,
// system box (insertion draws) and the last call's energy change.
constexpr int kBatchMaxBuf = 8;
struct RepBuf {
  int ibfftyp, qbias, nat, ntotat, ninsert, nremove;
  double avnum, mu, kb, lzmin, lzmax, rmin, rmax;
};
struct RepGc {
  int nb, n, shape, err;  // err: a kErr* flag of this replica's last call
  double lx, ly, lz, cx, cy, cz, rsphe2, iecx, iecy;
  double dener;
  RepBuf buf[kBatchMaxBuf];
};

// gcmc.cu: ngcmc attempts on every replica, one block each, FP64 ΔE
// (INTERACT on the float-float records); ibuf: each slot's buffer (0 none).
void launch_batch_grand(const KP &p, const RepDev *rep, RepGc *gc, int *ibuf, int nrep,
                        uint32_t mask, const uint64_t *seeds, uint64_t cycle, int ngcmc,
                        cudaStream_t stream);

void launch_batch_count(const KP &p, const RepDev *rep, RepGc *gc, int *ibuf, int nrep,
                        cudaStream_t stream);

// fields.cu: the FP32 field terms of every live slot (one warp each); lane
// 0 leaves (ememb, egsbpa, evdwgd, erfpar self) of the slot in pe.
void launch_batch_fields(const KP &p, const int *rep_of, const RepDev *rep, float4 *pe,
                         int nslots, uint32_t mask, int qforces, cudaStream_t stream);

}  // namespace bgpu
