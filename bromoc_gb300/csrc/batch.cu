// Replica batches on the device: many independent systems of uneven size
// advance together.
//
//   k_batch_fields (fields.cu): the FP32 field terms of every live slot.
//   k_batch_pairs: every tile pair of every replica, one warp each, through
//                  the Newton-3 pair tile of the single-system kernels
//                  (pairs_n3.cuh) on that replica's slots; partial forces
//                  per tile pair into the replica's stretch of the buffers.
//   k_batch_asm:   one block per tile of 32 ions of one replica: the tile
//                  assembly and dynamics0 move of the single-system path
//                  (move32.cuh) with the replica's box and noise key, in
//                  place (the pair launch has finished reading positions).
//
// Replicas fall into size buckets (fewer than 1000 ions, up to 4000, more);
// each bucket's tile pairs and tiles are launched separately, with the pair
// kernel's warps per block chosen for that bucket by an autotuner (timed
// pair passes, which change no state, at the first BD step after the
// replicas change).  A run of BD steps -- the upload of the seeds and of
// the step index, then every step's launches -- is captured once into a
// CUDA graph and replayed for later calls with the same step count: one
// graph launch per call.  The kernels read the step index from device
// memory, so one graph serves every step0.
//
// A replica's particles, partial sums and moves are exactly those of a
// single context holding that replica (same summation order, noise drawn
// from the replica's seed with the single context's counters), so a batch
// replica follows the trajectory of bromoc_gpu_bd_steps bit for bit.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bromoc_gpu.h"
#include "batch.cuh"
#include "ff.cuh"
#include "launch.h"
#include "move32.cuh"
#include "pairs_n3.cuh"
#include "physics.cuh"

namespace bgpu {

constexpr int kAsmTileWarps = 16;  // as the single-system tile assembly (same sums)
// replica size buckets: [0, 1000), [1000, 4000], above
constexpr int kBuckets = 3;
inline int size_bucket(int n) { return n < 1000 ? 0 : (n <= 4000 ? 1 : 2); }
// the autotuner's candidates for the pair kernel's warps per block
constexpr int kPairWarpChoices[3] = {2, 4, 8};

// Energies of one tile pair: ecoul, elj, esrpmf, eefpot, RFPAR cross.
constexpr int kRowTerms = 5;

// work / wpart: one bucket's stretch of the work list and its energy slots
template <bool RF, int W>
__global__ void __launch_bounds__(32 * W)
    k_batch_pairs(const __grid_constant__ KP p, const RepDev *rep, const int2 *work, int nwork,
                  float4 *tpf, float *tpb, float *wpart) {
  __shared__ N3Warp<RF> nw[W];
  __shared__ float4 tab[kIpqMax];
  const int nt = p.nion_t;
  for (int k = threadIdx.x; k < nt * ipq_stride(nt); k += blockDim.x) tab[k] = __ldg(p.ipq + k);
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int widx = blockIdx.x * W + w;
  if (widx >= nwork) return;  // no block-wide barrier follows
  const int2 wk = work[widx];
  const RepDev &R = rep[wk.x];
  const PairSys ps{p.pk1 + R.off, p.pk2 + R.off, p.pk3 + R.off, tpf + (size_t)R.poff * 64,
                   tpb + (size_t)R.poff * 64, 0, 0, R.n, (R.n + 31) >> 5, R.rows};
  float e[kRowTerms] = {0.f, 0.f, 0.f, 0.f, 0.f};
  n3_tile<true, RF, false>(p, ps, wk.y, 1, nw[w], tab, e);
  e[1] *= 1.0f / 6.0f;  // the tile sums 6 x elj
  // the tile pair's energies -> its slot (fixed shuffle tree)
#pragma unroll
  for (int k = 0; k < kRowTerms; ++k) {
    float v = e[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) wpart[(size_t)widx * kRowTerms + k] = v;
  }
}

// One block per (replica, tile): the tile assembly and move of the single
// system path on the replica's slots; fout (if not moving): 3 doubles per
// slot.
// step: *step0 + k (the step index lives in device memory for graph replay)
template <bool RF>
__global__ void __launch_bounds__(32 * kAsmTileWarps, 2)
    k_batch_asm(const __grid_constant__ KP p, const RepDev *rep, const int2 *tiles,
                const float4 *tpf, const float *tpb, int do_bd, const uint64_t *step0, int k,
                double *fout) {
  __shared__ float part[kAsmTileWarps][10][32];
  const uint64_t step = *step0 + (uint64_t)k;
  const int2 tk = tiles[blockIdx.x];
  const RepDev &R = rep[tk.x];
  const size_t o = R.off;
  const AsmSys ms{p.pk1 + o, p.pk2 + o, p.pk3 + o, p.typei + o, p.ffield_f + o, nullptr,
                  p.rfd + 2 * o,
                  tpf + (size_t)R.poff * 64, tpb + (size_t)R.poff * 64, p.cap, 0, 0, R.n,
                  (R.n + 31) >> 5, R.seed, &R.box,
                  fout ? fout + 3 * o : nullptr, fout ? fout + 3 * o + 1 : nullptr,
                  fout ? fout + 3 * o + 2 : nullptr, 3};
  AssembleFlags fl{};
  fl.fp32_partials = 1;
  fl.ntile = ms.T;
  fl.rf_ab = RF;
  assemble_tile<kAsmTileWarps>(p, ms, fl, do_bd, 0, step, tk.y, 0, part);
}

// Per-replica ENERGY terms (energy.mono.f90 slots) from the field terms of
// its slots and the pair terms of its work items; one block per replica,
// fixed-order sums in FP64.
__global__ void __launch_bounds__(256)
    k_batch_ereduce(const RepDev *rep, const float4 *pe, const float *wpart, int rfpar_on,
                    double *eterms) {
  __shared__ double red[(256 / 32) * 9];
  __shared__ double tot[9];
  const RepDev &R = rep[blockIdx.x];
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = threadIdx.x; k < R.n; k += blockDim.x) {
    const float4 q = pe[R.off + k];
    v[0] += q.x;
    v[1] += q.y;
    v[2] += q.z;
    v[3] += q.w;
  }
  for (int k = R.w0 + threadIdx.x; k < R.w1; k += blockDim.x)
    for (int m = 0; m < kRowTerms; ++m) v[4 + m] += wpart[(size_t)k * kRowTerms + m];
  block_sum<9>(v, red, tot);
  if (threadIdx.x == 0) {
    double o[kNTerms] = {};
    o[9] = tot[0];              // ememb
    o[10] = tot[1];             // egsbpa
    o[12] = tot[2];             // evdwgd
    o[13] = tot[3] + tot[8];    // erfpar: self + cross
    o[1] = tot[4];              // eelec
    o[2] = tot[5];              // evdw
    o[3] = tot[6];              // esrpmf
    o[4] = tot[7];              // eefpot
    o[11] = rfpar_on ? o[13] : 0.0;
    o[0] = o[9] + o[10] + o[12] + o[13] + o[1] + o[2] + o[3] + o[4];
    for (int k = 0; k < kNTerms; ++k) eterms[(size_t)blockIdx.x * kNTerms + k] = o[k];
  }
}

}  // namespace bgpu

using namespace bgpu;

struct bromoc_batch {
  bromoc_ctx *proto = nullptr;
  KP kp{};                     // prototype's parameter block, batch arrays swapped in
  cudaStream_t stream = nullptr;
  std::string err;
  int nrep = 0, nslots = 0, nwork = 0, cur = 0;  // cur: always 0 (moves are in place)
  // buckets: work items [wb[k], wb[k+1]) and tiles [tb[k], tb[k+1]) of bucket k
  int wb[kBuckets + 1] = {}, tb[kBuckets + 1] = {};
  int pair_warps[kBuckets] = {4, 4, 4};  // the autotuner's choice per bucket
  float tune_ms[kBuckets][3] = {};       // its measured pair pass per candidate
  bool tuned = false;
  // graph of a run of BD steps: replayed while nsteps and rf match
  bool use_graph = true;
  cudaGraphExec_t gexec = nullptr;
  int g_nsteps = -1, g_rf = -1, g_terms = -1;
  long long g_launches = 0;      // kernels in the graph
  long long graph_launches = 0;  // graph launches so far
  uint64_t *step_pinned = nullptr, *d_step0 = nullptr;
  std::vector<int> cap, off, n;
  std::vector<RepDev> rep_h;   // host copy of the replica records
  std::vector<int> nwtype_h;   // [ntype+1] ion type -> combined type
  std::vector<double> cg_h;    // [ntype+1] charges
  bool have_sys = false;
  int orphaned = 0;  // set when the prototype context is destroyed first
  // device
  RepDev *rep = nullptr;
  int *rep_of = nullptr;
  int2 *work = nullptr;    // (replica, tile pair), replica by replica
  int2 *tiles = nullptr;   // (replica, tile)
  int ntiles = 0, ntile_cap = 0;
  float4 *tpf = nullptr;   // per-tile-pair partials, replica r from poff_r * 64
  float *tpb = nullptr;
  float4 *pk1[2] = {nullptr, nullptr}, *pk2[2] = {nullptr, nullptr};
  float4 *pe = nullptr;
  float *wpart = nullptr;
  double *eterms = nullptr;
  RepDev *rep_pinned = nullptr;
  // GCMC of the replicas (bromoc_batch_grand)
  std::vector<RepGc> gc_h;
  RepGc *gc = nullptr;
  int *ibuf = nullptr;         // [nslots] buffer of each slot (0 none)
  uint64_t *d_seeds = nullptr; // [nrep]
  bool have_buffers = false;
  std::vector<void *> allocs;
  long long launches = 0;
};

namespace {

int bset(bromoc_batch *b, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCU(call)                                                              \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return bset(b, BROMOC_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
  } while (0)

template <class T>
int balloc(bromoc_batch *b, T **p, size_t count) {
  *p = nullptr;
  cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess)
    return bset(b, BROMOC_E_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                cudaGetErrorString(e));
  b->allocs.push_back((void *)*p);
  return BROMOC_OK;
}

void split(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

void drop_graph(bromoc_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_nsteps = b->g_rf = -1;
}

// work items: every pair-tile item (replica, n3_item index) and every tile
// (replica, t) of the live particles, bucket by bucket and replica by
// replica within a bucket; w0, w1 bound each replica's pair-tile items
int rebuild_work(bromoc_batch *b, bool retune = true) {
  std::vector<int2> items, tiles;
  for (int k = 0; k < kBuckets; ++k) {
    b->wb[k] = (int)items.size();
    b->tb[k] = (int)tiles.size();
    for (int r = 0; r < b->nrep; ++r) {
      if (size_bucket(b->n[r]) != k) continue;
      const int T = (b->n[r] + 31) / 32;
      b->rep_h[r].w0 = (int)items.size();
      b->rep_h[r].rows = n3_rows(T);
      for (int q = 0; q < n3_work(T, b->rep_h[r].rows); ++q) items.push_back(make_int2(r, q));
      b->rep_h[r].w1 = (int)items.size();
      for (int t = 0; t < T; ++t) tiles.push_back(make_int2(r, t));
    }
  }
  b->wb[kBuckets] = (int)items.size();
  b->tb[kBuckets] = (int)tiles.size();
  if (retune) b->tuned = false;
  drop_graph(b);
  if ((int)items.size() > b->nwork) {
    if (b->work) cudaFree(b->work);
    if (b->wpart) cudaFree(b->wpart);
    b->work = nullptr;
    b->wpart = nullptr;
    BCU(cudaMalloc((void **)&b->work, items.size() * sizeof(int2)));
    BCU(cudaMalloc((void **)&b->wpart, items.size() * kRowTerms * sizeof(float)));
  }
  b->nwork = (int)items.size();
  if ((int)tiles.size() > b->ntile_cap) {
    if (b->tiles) cudaFree(b->tiles);
    b->tiles = nullptr;
    BCU(cudaMalloc((void **)&b->tiles, tiles.size() * sizeof(int2)));
    b->ntile_cap = (int)tiles.size();
  }
  b->ntiles = (int)tiles.size();
  if (!items.empty())
    BCU(cudaMemcpy(b->work, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice));
  if (!tiles.empty())
    BCU(cudaMemcpy(b->tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
  BCU(cudaMemcpy(b->rep, b->rep_h.data(), b->nrep * sizeof(RepDev), cudaMemcpyHostToDevice));
  return BROMOC_OK;
}

template <bool RF>
void launch_pairs_w(int w, int nb, cudaStream_t s, const KP &p, const RepDev *rep,
                    const int2 *work, int nwork, float4 *tpf, float *tpb, float *wpart) {
  if (w == 2)
    k_batch_pairs<RF, 2><<<nb, 64, 0, s>>>(p, rep, work, nwork, tpf, tpb, wpart);
  else if (w == 8)
    k_batch_pairs<RF, 8><<<nb, 256, 0, s>>>(p, rep, work, nwork, tpf, tpb, wpart);
  else
    k_batch_pairs<RF, 4><<<nb, 128, 0, s>>>(p, rep, work, nwork, tpf, tpb, wpart);
}

// The pair launch of bucket k with w warps per block.
void launch_bucket_pairs(bromoc_batch *b, const KP &p, bool rf, int k, int w) {
  const int n = b->wb[k + 1] - b->wb[k];
  if (n <= 0) return;
  const int nb = (n + w - 1) / w;
  const int2 *work = b->work + b->wb[k];
  float *wpart = b->wpart + (size_t)b->wb[k] * kRowTerms;
  if (rf)
    launch_pairs_w<true>(w, nb, b->stream, p, b->rep, work, n, b->tpf, b->tpb, wpart);
  else
    launch_pairs_w<false>(w, nb, b->stream, p, b->rep, work, n, b->tpf, b->tpb, wpart);
  b->launches += 1;
}

// The pair and assembly launches of one step, bucket by bucket (do_bd:
// move, else forces into fout if given); kstep: the step's offset from the
// device-resident step index.
void launch_pairs_asm(bromoc_batch *b, const KP &p, bool rf, int do_bd, int kstep,
                      double *fout) {
  for (int k = 0; k < kBuckets; ++k) launch_bucket_pairs(b, p, rf, k, b->pair_warps[k]);
  for (int k = 0; k < kBuckets; ++k) {
    const int nt = b->tb[k + 1] - b->tb[k];
    if (nt <= 0) continue;
    const int2 *tiles = b->tiles + b->tb[k];
    if (rf)
      k_batch_asm<true><<<nt, 32 * kAsmTileWarps, 0, b->stream>>>(
          p, b->rep, tiles, b->tpf, b->tpb, do_bd, b->d_step0, kstep, fout);
    else
      k_batch_asm<false><<<nt, 32 * kAsmTileWarps, 0, b->stream>>>(
          p, b->rep, tiles, b->tpf, b->tpb, do_bd, b->d_step0, kstep, fout);
    b->launches += 1;
  }
}

// The autotuner: per bucket, every candidate warps-per-block of the pair
// kernel timed over three pair passes (after one untimed pass) with CUDA
// events on the batch's stream; the fastest is kept.  A pair pass only
// writes the partial buffers, which the next step rewrites, so tuning moves
// no particle.
int autotune(bromoc_batch *b, const KP &p, bool rf) {
  cudaEvent_t e0, e1;
  BCU(cudaEventCreate(&e0));
  BCU(cudaEventCreate(&e1));
  const long long l0 = b->launches;
  for (int k = 0; k < kBuckets; ++k) {
    if (b->wb[k + 1] == b->wb[k]) continue;
    float best = 0.0f;
    for (int c = 0; c < 3; ++c) {
      const int w = kPairWarpChoices[c];
      launch_bucket_pairs(b, p, rf, k, w);
      cudaEventRecord(e0, b->stream);
      for (int rep = 0; rep < 3; ++rep) launch_bucket_pairs(b, p, rf, k, w);
      cudaEventRecord(e1, b->stream);
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      b->tune_ms[k][c] = ms / 3.0f;
      if (c == 0 || ms < best) {
        best = ms;
        b->pair_warps[k] = w;
      }
    }
  }
  b->launches = l0;  // tuning passes are not steps
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  BCU(cudaGetLastError());
  b->tuned = true;
  return BROMOC_OK;
}

// The launches of nsteps BD steps with their uploads (seeds in the replica
// records, the step index), in stream order.
void enqueue_steps(bromoc_batch *b, const KP &p, bool rf, uint32_t terms, int nsteps) {
  cudaMemcpyAsync(b->rep, b->rep_pinned, b->nrep * sizeof(RepDev), cudaMemcpyHostToDevice,
                  b->stream);
  cudaMemcpyAsync(b->d_step0, b->step_pinned, sizeof(uint64_t), cudaMemcpyHostToDevice,
                  b->stream);
  for (int k = 0; k < nsteps; ++k) {
    launch_batch_fields(p, b->rep_of, b->rep, b->pe, b->nslots, terms, 1, b->stream);
    b->launches += 1;
    launch_pairs_asm(b, p, rf, 1, k, nullptr);
  }
}

}  // namespace

extern "C" {

int bromoc_batch_create(bromoc_ctx *proto, int32_t nrep, const int32_t *capacity,
                        bromoc_batch **out) {
  if (!proto || !out || nrep < 1 || !capacity) return BROMOC_E_ARG;
  *out = nullptr;
  const KP *pk = nullptr;
  cudaStream_t stream = nullptr;
  int rc = bromoc_ctx_prepare_f32(proto, &pk, &stream);
  if (rc) return rc;
  if (!pk->ipq_ok)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE,
                           "batch: needs analytic ion-ion laws (no EFPOT) and <= 16 ion types");
  if (pk->periodic)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "batch: the periodic mode is not supported");
  if (pk->nsites != 0)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "batch: replicas hold ions only (no sites)");
  if (pk->mm.on)
    return bromoc_ctx_fail(proto, BROMOC_E_STATE, "batch: the MMIJ reaction field is not supported");
  bromoc_batch *b = new bromoc_batch;
  b->proto = proto;
  b->kp = *pk;
  b->stream = stream;
  bromoc_ctx_attach(proto, &b->orphaned);
  b->nrep = nrep;
  b->cap.resize(nrep);
  b->off.resize(nrep);
  b->n.assign(nrep, 0);
  b->rep_h.assign(nrep, RepDev{});
  int slots = 0;
  size_t npair = 0;
  for (int r = 0; r < nrep; ++r) {
    if (capacity[r] < 1) {
      delete b;
      return bromoc_ctx_fail(proto, BROMOC_E_ARG, "batch: every capacity must be >= 1");
    }
    b->off[r] = slots;
    b->cap[r] = capacity[r];
    b->rep_h[r].off = slots;
    b->rep_h[r].cap = capacity[r];
    b->rep_h[r].poff = (int)npair;
    slots += (capacity[r] + 31) / 32 * 32;  // replicas start on tile boundaries
    npair += n3_pairs((capacity[r] + 31) / 32);
  }
  b->nslots = slots;
  KP &p = b->kp;
  const size_t ns = slots;
  rc = balloc(b, &b->rep, nrep);
  if (!rc) rc = balloc(b, &b->rep_of, ns);
  if (!rc) rc = balloc(b, &b->pk1[0], ns);
  if (!rc) rc = balloc(b, &b->pk2[0], ns);
  float4 *pk3 = nullptr, *rfd = nullptr;
  float *ffield = nullptr;
  int *typei = nullptr;
  DevState *st = nullptr;
  if (!rc) rc = balloc(b, &pk3, ns);
  if (!rc) rc = balloc(b, &rfd, 2 * ns);
  if (!rc) rc = balloc(b, &ffield, 3 * ns);
  if (!rc) rc = balloc(b, &typei, ns);
  if (!rc) rc = balloc(b, &b->pe, ns);
  if (!rc) rc = balloc(b, &b->eterms, (size_t)nrep * kNTerms);
  if (!rc) rc = balloc(b, &b->tpf, npair * 64);
  if (!rc) rc = balloc(b, &b->tpb, npair * 64);
  if (!rc) rc = balloc(b, &st, 1);
  if (!rc) rc = balloc(b, &b->d_step0, 1);
  double2 *gcrf = nullptr;
  if (!rc) rc = balloc(b, &b->gc, nrep);
  if (!rc) rc = balloc(b, &b->ibuf, ns);
  if (!rc) rc = balloc(b, &b->d_seeds, nrep);
  if (!rc) rc = balloc(b, &gcrf, ns);
  if (!rc && cudaMallocHost((void **)&b->rep_pinned, nrep * sizeof(RepDev)) != cudaSuccess)
    rc = bset(b, BROMOC_E_NOMEM, "batch: pinned replica records");
  if (!rc && cudaMallocHost((void **)&b->step_pinned, sizeof(uint64_t)) != cudaSuccess)
    rc = bset(b, BROMOC_E_NOMEM, "batch: pinned step index");
  if (rc) {
    const std::string msg = b->err;
    bromoc_batch_destroy(b);
    return bromoc_ctx_fail(proto, rc, msg.c_str());
  }
  std::vector<int> rep_of(ns, 0);
  for (int r = 0; r < nrep; ++r)
    for (int k = b->off[r]; k < (r + 1 < nrep ? b->off[r + 1] : slots); ++k) rep_of[k] = r;
  cudaMemcpy(b->rep_of, rep_of.data(), ns * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemset(pk3, 0, ns * sizeof(float4));
  cudaMemset(b->pk1[0], 0, ns * sizeof(float4));
  cudaMemset(b->pk2[0], 0, ns * sizeof(float4));
  cudaMemset(st, 0, sizeof(DevState));
  cudaMemset(b->ibuf, 0, ns * sizeof(int));
  cudaMemset(gcrf, 0, ns * sizeof(double2));
  b->gc_h.assign(nrep, RepGc{});
  // host copies of the type tables
  b->nwtype_h.resize(p.ntype + 1);
  b->cg_h.resize(p.ntype + 1);
  cudaMemcpy(b->nwtype_h.data(), p.nwtype, (p.ntype + 1) * sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(b->cg_h.data(), p.cg, (p.ntype + 1) * sizeof(double), cudaMemcpyDeviceToHost);
  // batch arrays in the parameter block
  p.cap = slots;
  p.nsites = 0;
  p.nfix = 0;
  p.st = st;
  p.pk3 = pk3;
  p.rfd = rfd;
  p.ffield_f = ffield;
  p.typei = typei;
  p.gc_rf = gcrf;
  p.qproxdiff = 0;
  p.qcountion = 0;  // no crossing counters in a batch
  int *warn = nullptr;
  if (balloc(b, &warn, p.nttyp + 1) == BROMOC_OK) cudaMemset(warn, 0, (p.nttyp + 1) * sizeof(int));
  p.warn = warn;
  if (cudaGetLastError() != cudaSuccess) {
    bromoc_batch_destroy(b);
    return bromoc_ctx_fail(proto, BROMOC_E_CUDA, "batch: setup copies failed");
  }
  if ((rc = rebuild_work(b))) {
    const std::string msg = b->err;
    bromoc_batch_destroy(b);
    return bromoc_ctx_fail(proto, rc, msg.c_str());
  }
  *out = b;
  return BROMOC_OK;
}

int bromoc_batch_destroy(bromoc_batch *b) {
  if (!b) return BROMOC_E_ARG;
  if (!b->orphaned) {
    if (b->stream) cudaStreamSynchronize(b->stream);
    bromoc_ctx_detach(b->proto, &b->orphaned);
  }
  for (void *a : b->allocs) cudaFree(a);
  if (b->work) cudaFree(b->work);
  if (b->wpart) cudaFree(b->wpart);
  if (b->tiles) cudaFree(b->tiles);
  if (b->rep_pinned) cudaFreeHost(b->rep_pinned);
  if (b->step_pinned) cudaFreeHost(b->step_pinned);
  drop_graph(b);
  delete b;
  cudaGetLastError();  // leave no non-sticky error behind for the next call
  return BROMOC_OK;
}

const char *bromoc_batch_last_error(const bromoc_batch *b) {
  return b ? b->err.c_str() : "null batch";
}

int64_t bromoc_batch_launch_count(const bromoc_batch *b) { return b ? b->launches : -1; }

}  // extern "C"

extern "C" {

int bromoc_batch_set_systems(bromoc_batch *b, const bromoc_system *sys) {
  if (!b || !sys) return bset(b, BROMOC_E_ARG, "set_systems: null");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  // the drift and noise factors are shared (prototype tables): every
  // replica must have the prototype's dt, kbt and bdmax
  for (int r = 0; r < b->nrep; ++r) {
    const bromoc_system &q = sys[r];
    if ((float)q.bdmax != b->kp.f.bdmax || (float)(q.dt / q.kbt) != b->kp.f.kbtdt)
      return bset(b, BROMOC_E_ARG, "set_systems: replica %d differs in dt, kbt or bdmax", r);
    BoxF &bx = b->rep_h[r].box;
    bx = BoxF{};
    bx.shape = q.shape;
    bx.rsphe = (float)q.rsphe;
    bx.rsphe2 = (float)(q.rsphe * q.rsphe);
    bx.iecx = q.shape == BROMOC_ECYL ? (float)(2.0 / q.lx) : 0.0f;
    bx.iecy = q.shape == BROMOC_ECYL ? (float)(2.0 / q.ly) : 0.0f;
    const double bd[6] = {q.cx - 0.5 * q.lx, q.cx + 0.5 * q.lx, q.cy - 0.5 * q.ly,
                          q.cy + 0.5 * q.ly, q.cz - 0.5 * q.lz, q.cz + 0.5 * q.lz};
    for (int k = 0; k < 6; ++k) split(bd[k], bx.bh[k], bx.bl[k]);
    const double c[3] = {q.cx, q.cy, q.cz};
    for (int k = 0; k < 3; ++k) split(c[k], bx.ch[k], bx.cl[k]);
    RepGc &g = b->gc_h[r];  // insert.f90 draws in FP64
    g.shape = q.shape;
    g.lx = q.lx;
    g.ly = q.ly;
    g.lz = q.lz;
    g.cx = q.cx;
    g.cy = q.cy;
    g.cz = q.cz;
    g.rsphe2 = q.rsphe * q.rsphe;
    g.iecx = q.shape == BROMOC_ECYL ? 2.0 / q.lx : 0.0;
    g.iecy = q.shape == BROMOC_ECYL ? 2.0 / q.ly : 0.0;
  }
  BCU(cudaStreamSynchronize(b->stream));
  BCU(cudaMemcpy(b->rep, b->rep_h.data(), b->nrep * sizeof(RepDev), cudaMemcpyHostToDevice));
  b->have_sys = true;
  return BROMOC_OK;
}

int bromoc_batch_set_particles(bromoc_batch *b, int32_t r, int32_t n, const double *x,
                               const double *y, const double *z, const int32_t *typei) {
  if (!b || !x || !y || !z || !typei) return bset(b, BROMOC_E_ARG, "set_particles: null");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  if (r < 0 || r >= b->nrep) return bset(b, BROMOC_E_ARG, "set_particles: no replica %d", r);
  if (n < 0 || n > b->cap[r])
    return bset(b, BROMOC_E_CAPACITY, "set_particles: %d ions exceed capacity %d", n, b->cap[r]);
  const KP &p = b->kp;
  std::vector<float4> h1(n), h2(n), h3(n);
  for (int i = 0; i < n; ++i) {
    const int t = typei[i] < 0 ? -typei[i] : typei[i];
    if (t <= p.nold || t > p.ntype)
      return bset(b, BROMOC_E_ARG, "set_particles: typei(%d) = %d is not an ion type", i + 1,
                  typei[i]);
    float xh, xl, yh, yl, zh, zl;
    split(x[i], xh, xl);
    split(y[i], yh, yl);
    split(z[i], zh, zl);
    int code = (b->nwtype_h[t] - 1) | (1 << 16);  // every batch ion is mobile
    float fcode;
    std::memcpy(&fcode, &code, sizeof fcode);
    int fl = 2;
    float ffl;
    std::memcpy(&ffl, &fl, sizeof ffl);
    h1[i] = make_float4(xh, yh, zh, fcode);
    h2[i] = make_float4(xl, yl, zl, 0.0f);
    h3[i] = make_float4(0.0f, (float)b->cg_h[t], ffl, 0.0f);
  }
  BCU(cudaStreamSynchronize(b->stream));
  const size_t o = b->off[r];
  if (n > 0) {
    BCU(cudaMemcpy(b->pk1[b->cur] + o, h1.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    BCU(cudaMemcpy(b->pk2[b->cur] + o, h2.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    BCU(cudaMemcpy(b->kp.pk3 + o, h3.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    BCU(cudaMemcpy(b->kp.typei + o, typei, n * sizeof(int), cudaMemcpyHostToDevice));
  }
  BCU(cudaMemset(b->ibuf + o, 0, (size_t)b->cap[r] * sizeof(int)));
  b->n[r] = n;
  b->rep_h[r].n = n;
  return rebuild_work(b);
}

int bromoc_batch_set_buffers(bromoc_batch *b, int32_t r, const bromoc_buffers *bu,
                             const int32_t *ibuffer) {
  if (!b || !bu) return bset(b, BROMOC_E_ARG, "set_buffers: null");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  if (r < 0 || r >= b->nrep) return bset(b, BROMOC_E_ARG, "set_buffers: no replica %d", r);
  const int nb = bu->nbuffer, n = b->n[r];
  if (nb < 1 || nb > kBatchMaxBuf)
    return bset(b, BROMOC_E_ARG, "set_buffers: 1..%d buffers per replica", kBatchMaxBuf);
  if (!bu->ibfftyp || !bu->avnum || !bu->mu || !bu->kb || !bu->lzmin || !bu->lzmax ||
      !bu->rmin || !bu->rmax || !bu->qbufferbias || !bu->nat || !bu->ntotat ||
      (n > 0 && !ibuffer))
    return bset(b, BROMOC_E_ARG, "set_buffers: null");
  RepGc &g = b->gc_h[r];
  g.nb = nb;
  for (int k = 0; k < nb; ++k) {
    const int t = bu->ibfftyp[k];
    if (t <= b->kp.nold || t > b->kp.ntype)
      return bset(b, BROMOC_E_ARG, "set_buffers: buffer %d holds no ion type", k + 1);
    RepBuf &q = g.buf[k];
    q = RepBuf{};
    q.ibfftyp = t;
    q.qbias = bu->qbufferbias[k] ? 1 : 0;
    q.nat = bu->nat[k];
    q.ntotat = bu->ntotat[k];
    q.avnum = bu->avnum[k];
    q.mu = bu->mu[k];
    q.kb = bu->kb[k];
    q.lzmin = bu->lzmin[k];
    q.lzmax = bu->lzmax[k];
    q.rmin = bu->rmin[k];
    q.rmax = bu->rmax[k];
  }
  for (int i = 0; i < n; ++i)
    if (ibuffer[i] < 0 || ibuffer[i] > nb)
      return bset(b, BROMOC_E_ARG, "set_buffers: ibuffer(%d) = %d out of range", i + 1,
                  ibuffer[i]);
  BCU(cudaStreamSynchronize(b->stream));
  if (n > 0)
    BCU(cudaMemcpy(b->ibuf + b->off[r], ibuffer, n * sizeof(int), cudaMemcpyHostToDevice));
  b->have_buffers = true;
  return BROMOC_OK;
}

int bromoc_batch_grand(bromoc_batch *b, uint32_t terms, int32_t ngcmc, const uint64_t *seeds,
                       uint64_t cycle, double *dener) {
  if (!b || !seeds) return bset(b, BROMOC_E_ARG, "grand: null");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  if (ngcmc < 0 || cycle < 1) return bset(b, BROMOC_E_ARG, "grand: bad ngcmc or cycle");
  if (!b->have_sys) return bset(b, BROMOC_E_STATE, "grand: set_systems first");
  for (int r = 0; r < b->nrep; ++r)
    if (b->gc_h[r].nb < 1)
      return bset(b, BROMOC_E_STATE, "grand: replica %d has no buffers (set_buffers)", r);
  if (ngcmc == 0) {
    if (dener)
      for (int r = 0; r < b->nrep; ++r) dener[r] = 0.0;
    return BROMOC_OK;
  }
  for (int r = 0; r < b->nrep; ++r) b->gc_h[r].n = b->n[r];
  BCU(cudaMemcpyAsync(b->gc, b->gc_h.data(), b->nrep * sizeof(RepGc), cudaMemcpyHostToDevice,
                      b->stream));
  BCU(cudaMemcpyAsync(b->d_seeds, seeds, b->nrep * sizeof(uint64_t), cudaMemcpyHostToDevice,
                      b->stream));
  KP p = b->kp;  // the batch's own records (the block keeps the prototype's)
  p.pk1 = b->pk1[b->cur];
  p.pk2 = b->pk2[b->cur];
  launch_batch_grand(p, b->rep, b->gc, b->ibuf, b->nrep, terms, b->d_seeds, cycle, ngcmc,
                     b->stream);
  ++b->launches;
  BCU(cudaGetLastError());
  BCU(cudaMemcpyAsync(b->gc_h.data(), b->gc, b->nrep * sizeof(RepGc), cudaMemcpyDeviceToHost,
                      b->stream));
  BCU(cudaStreamSynchronize(b->stream));
  bool changed = false;
  int err = 0;
  for (int r = 0; r < b->nrep; ++r) {
    err |= b->gc_h[r].err;
    if (b->gc_h[r].n != b->n[r]) {
      b->n[r] = b->gc_h[r].n;
      b->rep_h[r].n = b->n[r];
      changed = true;
    }
    if (dener) dener[r] = b->gc_h[r].dener;
  }
  if (changed) {
    const int rc = rebuild_work(b, false);  // new counts; the per-bucket tuning stands
    if (rc) return rc;
  }
  if (err & kErrCapacity)
    return bset(b, BROMOC_E_CAPACITY, "grand: an insertion would exceed a replica's capacity");
  if (err) return bset(b, BROMOC_E_DEVICE, "grand: device error flags 0x%x", err);
  return BROMOC_OK;
}

int bromoc_batch_count(bromoc_batch *b) {
  if (!b) return BROMOC_E_ARG;
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  if (!b->have_buffers) return BROMOC_OK;
  for (int r = 0; r < b->nrep; ++r) {
    b->gc_h[r].n = b->n[r];
    b->gc_h[r].err = 0;
  }
  BCU(cudaMemcpyAsync(b->gc, b->gc_h.data(), b->nrep * sizeof(RepGc), cudaMemcpyHostToDevice,
                      b->stream));
  KP p = b->kp;
  p.pk1 = b->pk1[b->cur];
  p.pk2 = b->pk2[b->cur];
  launch_batch_count(p, b->rep, b->gc, b->ibuf, b->nrep, b->stream);
  ++b->launches;
  BCU(cudaGetLastError());
  BCU(cudaMemcpyAsync(b->gc_h.data(), b->gc, b->nrep * sizeof(RepGc), cudaMemcpyDeviceToHost,
                      b->stream));
  BCU(cudaStreamSynchronize(b->stream));
  for (int r = 0; r < b->nrep; ++r)
    if (b->gc_h[r].err & kErrOutside)
      return bset(b, BROMOC_E_DEVICE, "count: replica %d has a buffer ion outside its system", r);
  return BROMOC_OK;
}

int bromoc_batch_get_buffers(bromoc_batch *b, int32_t r, int32_t *nat, int32_t *ninsert,
                             int32_t *nremove, int32_t *typei, int32_t *ibuffer) {
  if (!b || r < 0 || r >= b->nrep) return bset(b, BROMOC_E_ARG, "get_buffers: bad replica");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  const RepGc &g = b->gc_h[r];
  for (int k = 0; k < g.nb; ++k) {
    if (nat) nat[k] = g.buf[k].nat;
    if (ninsert) ninsert[k] = g.buf[k].ninsert;
    if (nremove) nremove[k] = g.buf[k].nremove;
  }
  const int m = b->n[r];
  BCU(cudaStreamSynchronize(b->stream));
  if (typei && m > 0)
    BCU(cudaMemcpy(typei, b->kp.typei + b->off[r], m * sizeof(int), cudaMemcpyDeviceToHost));
  if (ibuffer && m > 0)
    BCU(cudaMemcpy(ibuffer, b->ibuf + b->off[r], m * sizeof(int), cudaMemcpyDeviceToHost));
  return BROMOC_OK;
}

int bromoc_batch_get_particles(bromoc_batch *b, int32_t r, int32_t *n, double *x, double *y,
                               double *z) {
  if (!b || r < 0 || r >= b->nrep) return bset(b, BROMOC_E_ARG, "get_particles: bad replica");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  const int m = b->n[r];
  if (n) *n = m;
  std::vector<float4> h1(m), h2(m);
  BCU(cudaStreamSynchronize(b->stream));
  if (m > 0) {
    BCU(cudaMemcpy(h1.data(), b->pk1[b->cur] + b->off[r], m * sizeof(float4),
                   cudaMemcpyDeviceToHost));
    BCU(cudaMemcpy(h2.data(), b->pk2[b->cur] + b->off[r], m * sizeof(float4),
                   cudaMemcpyDeviceToHost));
  }
  for (int i = 0; i < m; ++i) {
    if (x) x[i] = (double)h1[i].x + (double)h2[i].x;
    if (y) y[i] = (double)h1[i].y + (double)h2[i].y;
    if (z) z[i] = (double)h1[i].z + (double)h2[i].z;
  }
  return BROMOC_OK;
}

// nsteps BD steps (ENERGY + dynamics0) of every replica; eterms, if given,
// receives nrep x 14 ENERGY terms of the last step's configuration.
int bromoc_batch_bd_steps(bromoc_batch *b, uint32_t terms, int32_t nsteps, const uint64_t *seeds,
                          uint64_t step0, double *eterms) {
  if (!b || !seeds || nsteps < 0) return bset(b, BROMOC_E_ARG, "bd_steps: bad arguments");
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  cudaGetLastError();  // a stale non-sticky error of an unrelated call
  if (!b->have_sys) return bset(b, BROMOC_E_STATE, "bd_steps: set_systems first");
  for (int r = 0; r < b->nrep; ++r) b->rep_h[r].seed = seeds[r];
  BCU(cudaStreamSynchronize(b->stream));  // the pinned records may still be in use
  std::memcpy(b->rep_pinned, b->rep_h.data(), b->nrep * sizeof(RepDev));
  *b->step_pinned = step0;
  const bool rf = (terms & BROMOC_M_RFPAR) && b->kp.qrfpar;
  KP p = b->kp;
  p.pk1 = b->pk1[b->cur];
  p.pk2 = b->pk2[b->cur];
  if (nsteps > 0 && !b->tuned) {
    BCU(cudaMemcpyAsync(b->rep, b->rep_pinned, b->nrep * sizeof(RepDev),
                        cudaMemcpyHostToDevice, b->stream));
    int rc = autotune(b, p, rf);
    if (rc) return rc;
  }
  if (nsteps > 0 && b->use_graph) {
    if (!b->gexec || b->g_nsteps != nsteps || b->g_rf != (int)rf ||
        (uint32_t)b->g_terms != terms) {
      drop_graph(b);
      cudaGraph_t g = nullptr;
      const long long l0 = b->launches;
      BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_steps(b, p, rf, terms, nsteps);
      const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
      if (ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bset(b, BROMOC_E_CUDA, "bd_steps: graph capture: %s", cudaGetErrorString(ec));
      }
      const cudaError_t ei = cudaGraphInstantiate(&b->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) {
        b->gexec = nullptr;
        return bset(b, BROMOC_E_CUDA, "bd_steps: graph instantiate: %s", cudaGetErrorString(ei));
      }
      b->g_launches = b->launches - l0;
      b->launches = l0;
      b->g_nsteps = nsteps;
      b->g_rf = (int)rf;
      b->g_terms = (int)terms;
    }
    BCU(cudaGraphLaunch(b->gexec, b->stream));
    b->launches += b->g_launches;
    b->graph_launches += 1;
  } else if (nsteps > 0) {
    enqueue_steps(b, p, rf, terms, nsteps);
  }
  BCU(cudaGetLastError());
  if (eterms && nsteps > 0) {
    k_batch_ereduce<<<b->nrep, 256, 0, b->stream>>>(b->rep, b->pe, b->wpart, rf ? 1 : 0,
                                                    b->eterms);
    b->launches += 1;
    BCU(cudaMemcpyAsync(eterms, b->eterms, (size_t)b->nrep * kNTerms * sizeof(double),
                        cudaMemcpyDeviceToHost, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
  }
  return BROMOC_OK;
}

// ENERGY of every replica at its current configuration: nrep x 14 terms and,
// if forces is given, 3 doubles per slot (replica r's ion k at slot off_r + k,
// off_r from bromoc_batch_offset).
int bromoc_batch_energy(bromoc_batch *b, uint32_t terms, double *forces, double *eterms) {
  if (!b) return BROMOC_E_ARG;
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  cudaGetLastError();  // a stale non-sticky error of an unrelated call
  const bool rf = (terms & BROMOC_M_RFPAR) && b->kp.qrfpar;
  KP p = b->kp;
  p.pk1 = b->pk1[b->cur];
  p.pk2 = b->pk2[b->cur];
  double *fdev = nullptr;
  if (forces) BCU(cudaMalloc((void **)&fdev, (size_t)b->nslots * 3 * sizeof(double)));
  launch_batch_fields(p, b->rep_of, b->rep, b->pe, b->nslots, terms, 1, b->stream);
  launch_pairs_asm(b, p, rf, 0, 0, fdev);  // no move: the step index is not read
  k_batch_ereduce<<<b->nrep, 256, 0, b->stream>>>(b->rep, b->pe, b->wpart, rf ? 1 : 0,
                                                  b->eterms);
  b->launches += 2;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && eterms)
    e = cudaMemcpyAsync(eterms, b->eterms, (size_t)b->nrep * kNTerms * sizeof(double),
                        cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess && forces)
    e = cudaMemcpyAsync(forces, fdev, (size_t)b->nslots * 3 * sizeof(double),
                        cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (fdev) cudaFree(fdev);
  if (e != cudaSuccess) return bset(b, BROMOC_E_CUDA, "batch energy: %s", cudaGetErrorString(e));
  return BROMOC_OK;
}

int bromoc_batch_set_graph(bromoc_batch *b, int32_t on) {
  if (!b) return BROMOC_E_ARG;
  if (b->orphaned) return bset(b, BROMOC_E_STATE, "the prototype context was destroyed");
  BCU(cudaStreamSynchronize(b->stream));
  b->use_graph = on != 0;
  if (!b->use_graph) drop_graph(b);
  return BROMOC_OK;
}

int bromoc_batch_tuning(const bromoc_batch *b, int32_t *warps, int32_t *items, double *ms) {
  if (!b) return BROMOC_E_ARG;
  for (int k = 0; k < kBuckets; ++k) {
    if (warps) warps[k] = b->tuned && b->wb[k + 1] > b->wb[k] ? b->pair_warps[k] : 0;
    if (items) items[k] = b->wb[k + 1] - b->wb[k];
    for (int c = 0; c < 3; ++c)
      if (ms) ms[3 * k + c] = b->tuned ? (double)b->tune_ms[k][c] : 0.0;
  }
  return BROMOC_OK;
}

int64_t bromoc_batch_graph_launches(const bromoc_batch *b) {
  return b ? b->graph_launches : -1;
}

int bromoc_batch_offset(const bromoc_batch *b, int32_t r) {
  return (b && r >= 0 && r < b->nrep) ? b->off[r] : -1;
}

int bromoc_batch_slots(const bromoc_batch *b) { return b ? b->nslots : -1; }

}  // extern "C"
