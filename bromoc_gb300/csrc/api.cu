// C ABI of the GB300 cg-gcmc-bd inner loop (include/bromoc_gpu.h).
//
// The context owns every device allocation and a KP parameter block whose
// pointers are passed by value to the kernels.  Module state uploaded by the
// set_* calls corresponds to what the reference's deck interpreter leaves in
// its Fortran modules; the particle arrays stay device-resident between
// calls, and GCMC edits them in place on the device.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bromoc_gpu.h"
#include "launch.h"

using namespace bgpu;

namespace {
constexpr int kMaxChunks = 64;
constexpr int kPairTile = 64;  // == kPairThreads of energy.cu
constexpr int kSMs = 152;
}  // namespace

struct bromoc_ctx {
  KP kp{};
  std::string err;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int precision = BROMOC_FP64;
  std::vector<void *> allocs;
  // host mirrors
  int ntype = 0, nold = 0, nttyp = 0, ndna = 0, ntc = 0, cnt = 0;
  int nbuffer = 0, cntpts = 0;
  bool have_sys = false, have_types = false, have_pairs = false;
  bromoc_system sys{};
  std::vector<double> diffusion;  // 1-based
  std::vector<int> site_map;      // per-site repulsion map (nmcden)
  int phiv_nmaps = 0;
  // live ntot bookkeeping (see ntot_ub)
  int ntot_known = 0;
  long long attempts_total = 0, attempts_at_known = 0;
  // pinned words: [0] ntot read back, [1] error word, [2..3] dener_sum,
  // [4] ntot uploaded (never a target of a pending read-back)
  int *h_ntot = nullptr;
  cudaEvent_t ev_ntot = nullptr;
  bool rb_pending = false;
  long long rb_attempts = 0;
  // scratch
  bool have_scratch = false;
  int nslot_cap = 0;
  int ipart_slots = 0;
  int tp_tiles = 0;  // tiles the Newton-3 partial buffers hold
  int cell_cap = 0;  // cells the cell-list arrays hold
  McState *mc = nullptr;  // Metropolis chain record (device)
  bool nuc_on = false;    // DNA bonded/Go term lists are set
  // per-cycle profiles (simul1.f90:476-509) and the .btr frame staging buffer
  bool prof_on = false;
  ProfArgs prof{};
  uint32_t *traj_w = nullptr;
  long long traj_cap = 0;
  std::vector<int *> dependents;  // orphan flags of batches and adjoint engines
  double *d_dener = nullptr;
  // last energy plan (for dynamics())
  AssembleFlags last_fl{};
  bool have_forces = false;
  // FP32 mode: which copy of the positions is current (both after a pack)
  bool ff_fresh = false, dbl_fresh = true;
  long long launches = 0;  // kernels launched by this context
  // diagnostic kernel timing: event pairs per kernel family
  bool timing = false;
  bool fused_bd = true;  // nsteps BD steps in one cooperative launch where supported
  std::vector<KTimer> tpool[BROMOC_K_NKINDS];
  int tused[BROMOC_K_NKINDS] = {};
};

namespace {

int set_err(bromoc_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CU(call)                                                             \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      return set_err(ctx, BROMOC_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// A double as the nearest float plus the nearest float of the remainder.
float2 ffsplit(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

template <class T>
int dalloc(bromoc_ctx *ctx, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
  if (e != cudaSuccess)
    return set_err(ctx, BROMOC_E_NOMEM, "cudaMalloc(%zu bytes): %s",
                   n * sizeof(T), cudaGetErrorString(e));
  ctx->allocs.push_back((void *)*p);
  return BROMOC_OK;
}

void dfree(bromoc_ctx *ctx, void *p) {
  if (!p) return;
  for (auto &a : ctx->allocs)
    if (a == p) {
      cudaFree(p);
      a = nullptr;
    }
}

// allocate (replacing a previous allocation) and copy n host elements
template <class T>
int upload(bromoc_ctx *ctx, T **dst, const T *src, size_t n) {
  if (*dst) dfree(ctx, (void *)*dst);
  int rc = dalloc(ctx, dst, n);
  if (rc) return rc;
  if (src && n) CU(cudaMemcpy((void *)*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return BROMOC_OK;
}

// copy into a fresh 1-based device array of n+1 elements
template <class T>
int upload1(bromoc_ctx *ctx, const T **dst, const T *src, int n, T fill = T()) {
  std::vector<T> v(n + 1, fill);
  if (src)
    for (int i = 0; i < n; ++i) v[i + 1] = src[i];
  T *d = const_cast<T *>(*dst);
  int rc = upload(ctx, &d, v.data(), v.size());
  *dst = d;
  return rc;
}

// Drops the DNA bonded/Go term lists (set_sites renumbers the sites).
void clear_nucl(bromoc_ctx *ctx) {
  NucDev &n = ctx->kp.nuc;
  for (const void *a : {(const void *)n.site, (const void *)n.par, (const void *)n.af,
                        (const void *)n.te, (const void *)n.tf, (const void *)n.csr_start,
                        (const void *)n.csr_ent, (const void *)n.csn, (const void *)n.ck,
                        (const void *)n.cc, (const void *)n.cf})
    dfree(ctx, const_cast<void *>(a));
  n = NucDev{};
  ctx->nuc_on = false;
}

// Drops the MMIJ reaction field.
void clear_mmij(bromoc_ctx *ctx) {
  MmijDev &m = ctx->kp.mm;
  for (const void *a : {(const void *)m.lst, (const void *)m.bnorm, (const void *)m.m,
                        (const void *)m.tab, (const void *)m.in, (const void *)m.ist,
                        (const void *)m.coefp, (const void *)m.coef, (const void *)m.coef2,
                        (const void *)m.mq, (const void *)m.rowe})
    dfree(ctx, const_cast<void *>(a));
  m = MmijDev{};
}

Grid3 make_grid(const bromoc_grid &g) {
  Grid3 r{};
  r.nclx = g.nclx;
  r.ncly = g.ncly;
  r.nclz = g.nclz;
  r.dcel = g.dcel;
  r.idcel = 1.0 / g.dcel;
  r.tranx = 0.5 * (g.nclx - 1) * g.dcel;  // readphi.f90:49-51
  r.trany = 0.5 * (g.ncly - 1) * g.dcel;
  r.tranz = 0.5 * (g.nclz - 1) * g.dcel;
  r.xbcen = g.xbcen;
  r.ybcen = g.ybcen;
  r.zbcen = g.zbcen;
  return r;
}

bool grid_ok(const bromoc_grid *g) {
  return g && g->nclx >= 2 && g->ncly >= 2 && g->nclz >= 2 && g->dcel > 0.0;
}

// Upper bound of the device-resident ntot, without a host round trip.
int ntot_ub(bromoc_ctx *c) {
  if (c->rb_pending && cudaEventQuery(c->ev_ntot) == cudaSuccess) {
    c->ntot_known = *c->h_ntot;
    c->attempts_at_known = c->rb_attempts;
    c->rb_pending = false;
  }
  long long ub = c->ntot_known + (c->attempts_total - c->attempts_at_known);
  return (int)std::min<long long>(ub, c->kp.cap);
}

int sync_ntot(bromoc_ctx *ctx) {
  CU(cudaMemcpyAsync(ctx->h_ntot, &ctx->kp.st->ntot, sizeof(int),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->ntot_known = *ctx->h_ntot;
  ctx->attempts_at_known = ctx->attempts_total;
  ctx->rb_pending = false;
  return BROMOC_OK;
}

void split_ff(double v, float &h, float &l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

// One axis of one grid for the float-float cell search; an unset grid gets
// bounds that no position satisfies.
void fill_axis(AxisF &A, const Grid3 &g, int axis, bool set, double ub, double lb) {
  A = AxisF{};
  if (!set || g.dcel <= 0.0) {
    A.ubh = -INFINITY;
    A.lbh = INFINITY;
    return;
  }
  const double tran = axis == 0 ? g.tranx : (axis == 1 ? g.trany : g.tranz);
  const double cen = axis == 0 ? g.xbcen : (axis == 1 ? g.ybcen : g.zbcen);
  split_ff(tran - cen, A.oh, A.ol);
  split_ff(g.dcel, A.dh, A.dl);
  A.idc = (float)g.idcel;
  split_ff(ub, A.ubh, A.ubl);
  split_ff(lb, A.lbh, A.lbl);
  A.ncl = axis == 0 ? g.nclx : (axis == 1 ? g.ncly : g.nclz);
}

// fixcoor constants of one system in float-float (shell_simul.f90:914-919).
void fill_box(const bromoc_system &q, BoxF &b) {
  b = BoxF{};
  b.shape = q.shape;
  b.rsphe = (float)q.rsphe;
  b.rsphe2 = (float)(q.rsphe * q.rsphe);
  b.iecx = q.shape == BROMOC_ECYL ? (float)(2.0 / q.lx) : 0.0f;
  b.iecy = q.shape == BROMOC_ECYL ? (float)(2.0 / q.ly) : 0.0f;
  const double bd[6] = {q.cx - 0.5 * q.lx, q.cx + 0.5 * q.lx, q.cy - 0.5 * q.ly,
                        q.cy + 0.5 * q.ly, q.cz - 0.5 * q.lz, q.cz + 0.5 * q.lz};
  for (int k = 0; k < 6; ++k) split_ff(bd[k], b.bh[k], b.bl[k]);
  const double c[3] = {q.cx, q.cy, q.cz};
  for (int k = 0; k < 3; ++k) split_ff(c[k], b.ch[k], b.cl[k]);
  const double L[3] = {q.lx, q.ly, q.lz};
  for (int k = 0; k < 3; ++k) split_ff(L[k], b.Lh[k], b.Ll[k]);
}

// Single-precision constants of the FP32 kernels (KP::f) from the FP64 state.
void fill_f32(bromoc_ctx *ctx) {
  KP &p = ctx->kp;
  F32C &f = p.f;
  const Grid3 *gs[3] = {&p.g1, &p.g2, &p.g3};
  const bool set[3] = {p.qphix != 0, p.qphiv != 0, p.qrfpar != 0};
  for (int m = 0; m < 3; ++m)
    for (int a = 0; a < 3; ++a) {
      const Grid3 &g = *gs[m];
      const double cen = a == 0 ? g.xbcen : (a == 1 ? g.ybcen : g.zbcen);
      const double tran = a == 0 ? g.tranx : (a == 1 ? g.trany : g.tranz);
      // in-map tests of staticf1.f90:64-68, vdwgd1trln.f90, vdwgd1spln.f90:52
      // (one cell narrower for the B-spline), rfpar.f90:80-85; repulsion z
      // between vzmin and vzmax
      const double mg = (m == 1 && !p.qtrln) ? g.dcel : 0.0;
      double ub = cen + tran - mg, lb = cen - tran + mg;
      if (m == 1 && a == 2) {
        ub = p.vzmax;
        lb = p.vzmin;
      }
      fill_axis(f.ax[3 * m + a], g, a, set[m], ub, lb);
    }
  for (int a = 0; a < 3; ++a) fill_axis(f.ax[9 + a], p.g2, a, set[1], 0.0, 0.0);
  f.celec = (float)p.celec;
  f.sqrfac = (float)p.sqrfac;
  f.thold8 = (float)p.thold8;
  f.thold27 = (float)p.thold27;
  f.kbtdt = (float)p.kbtdt;
  f.bdmax = (float)p.bdmax;
  f.fact0n1 = (float)p.fact0n1;
  f.fact0n2 = (float)p.fact0n2;
  fill_box(ctx->sys, f.box);
  f.box.periodic = p.periodic;
  const double L[3] = {p.lx, p.ly, p.lz};
  for (int k = 0; k < 3; ++k) {
    f.L[k] = (float)L[k];
    f.iL[k] = (float)(1.0 / L[k]);
  }
  f.rc2 = (float)p.rc2;
}

int ensure_scratch(bromoc_ctx *ctx) {
  if (ctx->have_scratch) return BROMOC_OK;
  KP &p = ctx->kp;
  const size_t cap = p.cap;
  int rc;
  if ((rc = dalloc(ctx, &p.ffield, 3 * cap))) return rc;
  if ((rc = dalloc(ctx, &p.fii, (size_t)kMaxChunks * 3 * cap))) return rc;
  if ((rc = dalloc(ctx, &p.fis, 3 * cap))) return rc;
  if ((rc = dalloc(ctx, &p.frf, (size_t)kMaxChunks * 3 * cap))) return rc;
  if (ctx->precision == BROMOC_FP32) {
    if ((rc = dalloc(ctx, &p.fii_f, (size_t)kMaxChunks * 3 * cap))) return rc;
    if ((rc = dalloc(ctx, &p.frf_f, (size_t)kMaxChunks * 3 * cap))) return rc;
    if ((rc = dalloc(ctx, &p.pk1, cap))) return rc;
    if ((rc = dalloc(ctx, &p.pk2, cap))) return rc;
    if ((rc = dalloc(ctx, &p.pk3, cap))) return rc;
    if ((rc = dalloc(ctx, &p.rfd, 2 * cap))) return rc;
    if ((rc = dalloc(ctx, &p.ffield_f, 3 * cap))) return rc;
    if ((rc = dalloc(ctx, &p.fis_f, 3 * cap))) return rc;
  }
  const int tiles = (int)((cap + kPairTile - 1) / kPairTile) + 1;
  // fields (one block per 4 particles) + ion-ion and RFPAR (tiles x chunks)
  // + ion-site (tiles)
  ctx->nslot_cap = fields_blocks((int)cap) + tiles * (2 * kMaxChunks + 4) + 8;
  if ((rc = dalloc(ctx, &p.epart, (size_t)ctx->nslot_cap * kNTerms))) return rc;
  // block partials of INTERACT (a double per block) and GRAND (kSpec per
  // block): enough for GRAND's widest grid, a lane per particle and attempt
  const int islots = std::max(tiles + 2, grand_slots((int)cap));
  if ((rc = dalloc(ctx, &p.ipart, (size_t)islots * kSpec))) return rc;
  if ((rc = dalloc(ctx, &p.ierr, (size_t)islots * kSpec))) return rc;
  ctx->ipart_slots = islots;
  if ((rc = dalloc(ctx, &p.gc_rf, cap))) return rc;
  if ((rc = dalloc(ctx, &p.gc_rff, cap))) return rc;
  if ((rc = dalloc(ctx, &p.tff, kSpec))) return rc;
  if ((rc = dalloc(ctx, &p.rf_srfe, cap))) return rc;
  if ((rc = dalloc(ctx, &p.rf_reff, cap))) return rc;
  if ((rc = dalloc(ctx, &p.rf_d1, 3 * cap))) return rc;
  if ((rc = dalloc(ctx, &p.rf_d2, 3 * cap))) return rc;
  if ((rc = dalloc(ctx, &p.rf_in, cap))) return rc;
  if ((rc = dalloc(ctx, &p.dids, 5 * cap))) return rc;
  CU(cudaMemset(p.dids, 0, 5 * cap * sizeof(double)));
  if ((rc = dalloc(ctx, &p.eterms, kNTerms))) return rc;
  if ((rc = dalloc(ctx, &p.trial, kSpec))) return rc;
  if ((rc = dalloc(ctx, &p.ground, 1))) return rc;
  if ((rc = dalloc(ctx, &ctx->d_dener, 1))) return rc;
  ctx->have_scratch = true;
  return BROMOC_OK;
}

// Next free event pair of a kernel family, or nullptr when timing is off.
KTimer *next_timer(bromoc_ctx *c, int kind) {
  if (!c->timing) return nullptr;
  std::vector<KTimer> &v = c->tpool[kind];
  if (c->tused[kind] == (int)v.size()) {
    KTimer t{};
    if (cudaEventCreate(&t.a) != cudaSuccess || cudaEventCreate(&t.b) != cudaSuccess)
      return nullptr;
    v.push_back(t);
  }
  return &v[c->tused[kind]++];
}

// Source chunking of the pair kernels: enough blocks for ~2 waves of the
// 152 SMs, chunks a multiple of the 128-particle tile.
// Source chunks of a target-tiled pair kernel: about eight two-warp blocks
// per SM.  fine: chunks of any length down to kMinChunk sources (the FP64
// kernels, where a pair costs ~100 FP64 operations on GB300's narrow FP64
// pipe and a small system would otherwise occupy a few SMs); else whole
// source tiles.
constexpr int kMinChunk = 4;
void chunking(int ntargets, int nsources, int &nchunk, int &chunk, bool fine = false) {
  if (ntargets <= 0 || nsources <= 0) {
    nchunk = 0;
    chunk = kPairTile;
    return;
  }
  const int tiles = (ntargets + kPairTile - 1) / kPairTile;
  const int stiles = (nsources + kPairTile - 1) / kPairTile;
  int want = (8 * kSMs + tiles - 1) / tiles;  // ~8 two-warp blocks per SM
  if (fine) {
    want = std::max(1, std::min(want, kMaxChunks));
    chunk = std::max(kMinChunk, (nsources + want - 1) / want);
  } else {
    want = std::max(1, std::min(std::min(want, stiles), kMaxChunks));
    chunk = ((stiles + want - 1) / want) * kPairTile;  // source tiles per chunk
  }
  nchunk = (nsources + chunk - 1) / chunk;
}

// Cells of the FP32 extension mode's cell list: the most cubes of edge at
// least rc (1 + 1e-4) along each box edge; false (no cell list) unless
// every axis holds four or more, where the 27 neighbour cells are a strict
// part of the box.
bool cell_grid(KP &p) {
  p.ncells = 0;
  if (!p.periodic || !(p.rc2 > 0.0)) return false;
  const double rc = std::sqrt(p.rc2) * (1.0 + 1e-4);
  const double L[3] = {p.lx, p.ly, p.lz};
  int n = 1;
  for (int a = 0; a < 3; ++a) {
    p.nc[a] = (int)std::floor(L[a] / rc);
    if (p.nc[a] < 4) return false;
    p.cinv[a] = (float)(p.nc[a] / L[a]);
    n *= p.nc[a];
  }
  p.ncells = n;
  return true;
}

int ensure_cells(bromoc_ctx *ctx) {
  KP &p = ctx->kp;
  int rc;
  if (!p.cell_ion) {
    if ((rc = dalloc(ctx, &p.cell_ion, (size_t)p.cap))) return rc;
    if ((rc = dalloc(ctx, &p.ion_cell, (size_t)p.cap))) return rc;
  }
  if (p.ncells > ctx->cell_cap) {
    CU(cudaStreamSynchronize(ctx->stream));
    dfree(ctx, p.cell_n);
    dfree(ctx, p.cell_start);
    p.cell_n = p.cell_start = nullptr;
    ctx->cell_cap = 0;
    if ((rc = dalloc(ctx, &p.cell_n, (size_t)p.ncells + 1))) return rc;
    if ((rc = dalloc(ctx, &p.cell_start, (size_t)p.ncells + 1))) return rc;
    ctx->cell_cap = p.ncells;
  }
  return BROMOC_OK;
}

int plan_energy(bromoc_ctx *ctx, uint32_t mask, bool reduce, EnergyPlan &plan,
                AssembleFlags &fl, bool timers = true) {
  KP &p = ctx->kp;
  plan.ntot_ub = ntot_ub(ctx);
  plan.fp32 = ctx->precision == BROMOC_FP32;
  plan.reduce_energy = reduce;
  const int nion = plan.ntot_ub - p.nsites;
  const int nmob = nion - p.nfix;
  fl = AssembleFlags{};
  fl.fp32_noise = plan.fp32;
  fl.fp32_partials = plan.fp32;
  plan.nuc = ctx->nuc_on && p.nsites > 0;
  plan.mmij = p.mm.on && (mask & BROMOC_M_MMIJ);
  fl.is = ((mask & BROMOC_M_NONBOND) && p.nsites > 0 && nion > 0) || plan.nuc;
  plan.ntile = p.ntile = 0;
  plan.cells = false;
  if (plan.fp32 && p.periodic && nion > 0 && pair_cfg32(p, plan.ntot_ub, mask).ntg > 0 &&
      cell_grid(p)) {  // extension mode: the cell-list pair kernel
    const int rc = ensure_cells(ctx);
    if (rc) return rc;
    plan.cells = true;
    plan.nchunk_ii = p.nchunk_ii = 1;
    plan.nchunk_rf = p.nchunk_rf = 0;
    fl.ii = 1;
    fl.ii_from = p.nsites + p.nfix;
    fl.nchunk_ii = 1;
  } else if (plan.fp32 && nion > 0 && (nion + 31) / 32 <= kN3MaxTiles &&
      pair_cfg32(p, plan.ntot_ub, mask).ntg > 0) {  // Newton-3 pair kernel
    const int T = (nion + 31) / 32;
    if (T > ctx->tp_tiles) {  // grow the tile-pair partials (rare)
      const int Ta = std::min(kN3MaxTiles, T + 8);
      CU(cudaStreamSynchronize(ctx->stream));
      dfree(ctx, p.tpf);
      dfree(ctx, p.tpb);
      p.tpf = nullptr;
      p.tpb = nullptr;
      ctx->tp_tiles = 0;
      int rc = dalloc(ctx, &p.tpf, (size_t)n3_pairs(Ta) * 64);
      if (!rc) rc = dalloc(ctx, &p.tpb, (size_t)n3_pairs(Ta) * 64);
      if (rc) return rc;
      ctx->tp_tiles = Ta;
    }
    plan.ntile = p.ntile = T;
    plan.nchunk_ii = plan.nchunk_rf = p.nchunk_ii = p.nchunk_rf = 0;
    fl.ntile = T;
    fl.rf_ab = pair_cfg32(p, plan.ntot_ub, mask).rf;
  } else if (plan.fp32 && p.periodic && pair_cfg32(p, plan.ntot_ub, mask).ntg > 0) {
    return set_err(ctx, BROMOC_E_CAPACITY,
                   "periodic mode in FP32: more than %d ions need at least four cells of "
                   "the cutoff along every box edge",
                   32 * kN3MaxTiles);
  } else if (plan.fp32) {  // one fused pair kernel (ion-ion + RFPAR cross)
    const PairCfg32 pc = pair_cfg32(p, plan.ntot_ub, mask);
    chunking(pc.ntg, nion, plan.nchunk_ii, p.chunk_ii);
    p.nchunk_ii = plan.nchunk_ii;
    plan.nchunk_rf = p.nchunk_rf = 0;
    fl.ii = pc.ntg > 0 && plan.nchunk_ii > 0;
    fl.ii_from = pc.t0;
    fl.nchunk_ii = fl.ii ? plan.nchunk_ii : 0;
  } else {
    chunking(nmob, nion, plan.nchunk_ii, p.chunk_ii, true);
    p.nchunk_ii = plan.nchunk_ii;
    chunking(nion, nion, plan.nchunk_rf, p.chunk_rf, true);
    p.nchunk_rf = plan.nchunk_rf;
    fl.ii = (mask & BROMOC_M_NONBOND) && nmob > 0 && plan.nchunk_ii > 0;
    fl.ii_from = p.nsites + p.nfix;
    fl.nchunk_ii = fl.ii ? plan.nchunk_ii : 0;
    fl.rf = (mask & BROMOC_M_RFPAR) && p.qrfpar && nion > 0 && plan.nchunk_rf > 0;
    fl.nchunk_rf = fl.rf ? plan.nchunk_rf : 0;
  }
  if (timers) {
    plan.t_pairs = (fl.ii || fl.ntile) ? next_timer(ctx, BROMOC_K_PAIRS) : nullptr;
    plan.t_rf = fl.rf ? next_timer(ctx, BROMOC_K_RFCROSS) : nullptr;
    plan.t_fields = plan.ntot_ub > 0 ? next_timer(ctx, BROMOC_K_FIELDS) : nullptr;
  }
  const int need = energy_slots(p, plan, mask);
  if (need > ctx->nslot_cap) {  // e.g. many DNA terms: grow the block partials
    CU(cudaStreamSynchronize(ctx->stream));
    dfree(ctx, p.epart);
    p.epart = nullptr;
    const int ncap = need + 64;
    int rc = dalloc(ctx, &p.epart, (size_t)ncap * kNTerms);
    if (rc) {
      ctx->nslot_cap = 0;
      return rc;
    }
    ctx->nslot_cap = ncap;
  }
  return BROMOC_OK;
}

int check_ready(bromoc_ctx *ctx) {
  // a non-sticky error of an earlier, unrelated runtime call would otherwise
  // be reported by this call's launch checks (faults stay sticky and are
  // still reported)
  cudaGetLastError();
  if (!ctx->have_sys || !ctx->have_types || !ctx->have_pairs)
    return set_err(ctx, BROMOC_E_STATE,
                   "set_system, set_types and set_pairs are required");
  if (ctx->kp.periodic && (ctx->kp.nsites > 0 || ctx->kp.qrfpar))
    return set_err(ctx, BROMOC_E_STATE, "periodic mode: ions only, without RFPAR");
  if (ctx->precision == BROMOC_FP32) fill_f32(ctx);
  return ensure_scratch(ctx);
}

// FP32 mode keeps the positions as float-float records while the per-step
// kernels run (they never read the FP64 arrays); these make one form current
// from the other.  No-ops in FP64 mode.
int ensure_ff(bromoc_ctx *ctx) {
  if (ctx->precision != BROMOC_FP32 || ctx->ff_fresh) return BROMOC_OK;
  launch_pack(ctx->kp, ntot_ub(ctx), true, ctx->stream);
  ctx->launches += 1;
  ctx->ff_fresh = true;
  CU(cudaGetLastError());
  return BROMOC_OK;
}

int ensure_dbl(bromoc_ctx *ctx) {
  if (ctx->precision != BROMOC_FP32 || ctx->dbl_fresh) return BROMOC_OK;
  launch_pack(ctx->kp, ntot_ub(ctx), false, ctx->stream);
  ctx->launches += 1;
  ctx->dbl_fresh = true;
  CU(cudaGetLastError());
  return BROMOC_OK;
}

// Turns a nonzero device error word (read back with the stream idle) into
// the API error, clearing the word and the guard record.
int device_err_result(bromoc_ctx *ctx, int e) {
  if (e) {
    int bad[3] = {0, 0, 0};
    CU(cudaMemcpy(bad, &ctx->kp.st->bad_site, sizeof bad, cudaMemcpyDeviceToHost));
    CU(cudaMemsetAsync(&ctx->kp.st->err, 0, 4 * sizeof(int), ctx->stream));
    if (e & kErrBarrier)  // every block passes launch_exit; clear the counters all the same
      CU(cudaMemsetAsync(&ctx->kp.st->bar_count, 0, 3 * sizeof(unsigned), ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    if (e == kErrCapacity)
      return set_err(ctx, BROMOC_E_CAPACITY, "grand: ntot is greater than capacity");
    if (e & kErrBarrier)
      return set_err(ctx, BROMOC_E_DEVICE,
                     "grand: a grid barrier timed out (flags 0x%x); the kernel returned early", e);
    return set_err(ctx, BROMOC_E_DEVICE,
                   "device error flags 0x%x (guard site %d: index %d, bound %d)", e,
                   bad[0], bad[1], bad[2]);
  }
  return BROMOC_OK;
}

int check_device_err(bromoc_ctx *ctx) {
  CU(cudaMemcpyAsync(ctx->h_ntot + 1, &ctx->kp.st->err, sizeof(int),
                     cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return device_err_result(ctx, ctx->h_ntot[1]);
}

}  // namespace

bool bromoc_ctx_pair_view(const bromoc_ctx *ctx, const KP **kp, cudaStream_t *stream,
                          int *precision) {
  if (!ctx || !ctx->have_sys || !ctx->have_types || !ctx->have_pairs) return false;
  *kp = &ctx->kp;
  *stream = ctx->stream;
  *precision = ctx->precision;
  return true;
}

int bromoc_ctx_prepare_f32(bromoc_ctx *ctx, const KP **kp, cudaStream_t *stream) {
  if (!ctx) return BROMOC_E_ARG;
  if (ctx->precision != BROMOC_FP32)
    return set_err(ctx, BROMOC_E_STATE, "batch: the prototype context must be FP32");
  const int rc = check_ready(ctx);
  if (rc) return rc;
  *kp = &ctx->kp;
  *stream = ctx->stream;
  return BROMOC_OK;
}

void bromoc_ctx_attach(bromoc_ctx *ctx, int *orphaned) {
  if (ctx && orphaned) ctx->dependents.push_back(orphaned);
}

void bromoc_ctx_detach(bromoc_ctx *ctx, int *orphaned) {
  if (!ctx) return;
  auto &d = ctx->dependents;
  d.erase(std::remove(d.begin(), d.end(), orphaned), d.end());
}

int bromoc_ctx_fail(bromoc_ctx *ctx, int code, const char *msg) {
  return set_err(ctx, code, "%s", msg);
}

extern "C" {

int bromoc_gpu_abi_version(void) { return BROMOC_ABI_VERSION; }

const char *bromoc_gpu_last_error(const bromoc_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "null context";
}

int bromoc_gpu_create(int32_t capacity, int32_t precision, void *stream,
                      bromoc_ctx **out) {
  if (!out) return BROMOC_E_ARG;
  *out = nullptr;
  if (capacity <= 0 || (precision != BROMOC_FP64 && precision != BROMOC_FP32))
    return BROMOC_E_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BROMOC_E_CUDA;
  bromoc_ctx *ctx = new bromoc_ctx();
  ctx->precision = precision;
  KP &p = ctx->kp;
  p.cap = capacity;
  p.celec = 1.60217656535E-19 * 1.60217656535E-19 /
            (4.0 * kPi * 8.854187817620E-12 * (4184.0 / 6.0221412927E23) * 1E-10);
  int rc = BROMOC_OK;
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
      rc = BROMOC_E_CUDA;
    ctx->own_stream = true;
  }
  if (!rc && cudaMallocHost((void **)&ctx->h_ntot, 8 * sizeof(int)) != cudaSuccess)
    rc = BROMOC_E_CUDA;
  if (!rc && cudaEventCreateWithFlags(&ctx->ev_ntot, cudaEventDisableTiming) != cudaSuccess)
    rc = BROMOC_E_CUDA;
  if (!rc) rc = dalloc(ctx, &p.st, 1);
  if (!rc) rc = dalloc(ctx, &p.x, capacity);
  if (!rc) rc = dalloc(ctx, &p.y, capacity);
  if (!rc) rc = dalloc(ctx, &p.z, capacity);
  if (!rc) rc = dalloc(ctx, &p.typei, capacity);
  if (!rc) rc = dalloc(ctx, &p.ibuffer, capacity);
  if (!rc) rc = dalloc(ctx, &p.fx, capacity);
  if (!rc) rc = dalloc(ctx, &p.fy, capacity);
  if (!rc) rc = dalloc(ctx, &p.fz, capacity);
  if (!rc && cudaMemset(p.st, 0, sizeof(DevState)) != cudaSuccess) rc = BROMOC_E_CUDA;
  if (!rc && cudaMemset(p.ibuffer, 0, capacity * sizeof(int)) != cudaSuccess) rc = BROMOC_E_CUDA;
  if (rc) {
    bromoc_gpu_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return BROMOC_OK;
}

int bromoc_gpu_destroy(bromoc_ctx *ctx) {
  if (!ctx) return BROMOC_OK;
  for (int *f : ctx->dependents) *f = 1;  // their stream and tables go now
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (void *a : ctx->allocs)
    if (a) cudaFree(a);
  for (auto &pool : ctx->tpool)
    for (KTimer &t : pool) {
      cudaEventDestroy(t.a);
      cudaEventDestroy(t.b);
    }
  if (ctx->h_ntot) cudaFreeHost(ctx->h_ntot);
  if (ctx->ev_ntot) cudaEventDestroy(ctx->ev_ntot);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BROMOC_OK;
}

int bromoc_gpu_set_system(bromoc_ctx *ctx, const bromoc_system *q) {
  if (!ctx || !q) return set_err(ctx, BROMOC_E_ARG, "set_system: null");
  if (q->kbt <= 0.0 || q->dt <= 0.0)
    return set_err(ctx, BROMOC_E_ARG, "set_system: kbt and dt must be positive");
  KP &p = ctx->kp;
  ctx->sys = *q;
  p.shape = q->shape;
  p.qcountion = q->qcountion;
  p.lx = q->lx;
  p.ly = q->ly;
  p.lz = q->lz;
  p.cx = q->cx;
  p.cy = q->cy;
  p.cz = q->cz;
  p.rsphe = q->rsphe;
  p.rsphe2 = q->rsphe * q->rsphe;
  p.iecx = q->shape == BROMOC_ECYL ? 2.0 / q->lx : 0.0;
  p.iecy = q->shape == BROMOC_ECYL ? 2.0 / q->ly : 0.0;
  p.lx2p = q->cx + 0.5 * q->lx;  // shell_simul.f90:914-919
  p.ly2p = q->cy + 0.5 * q->ly;
  p.lz2p = q->cz + 0.5 * q->lz;
  p.lx2m = q->cx - 0.5 * q->lx;
  p.ly2m = q->cy - 0.5 * q->ly;
  p.lz2m = q->cz - 0.5 * q->lz;
  p.ikbt = 1.0 / q->kbt;
  p.kbtdt = q->dt * p.ikbt;  // simul1.f90:342
  p.dt = q->dt;
  p.bdmax = q->bdmax;
  ctx->have_sys = true;
  if (ctx->have_types) {  // fact1a/fact2a depend on both (simul1.f90:345-348)
    std::vector<double> f1(ctx->ntype + 1, 0.0), f2(ctx->ntype + 1, 0.0);
    for (int i = 1; i <= ctx->ntype; ++i) {
      f1[i] = ctx->diffusion[i] * p.kbtdt;
      f2[i] = std::sqrt(2.0 * q->dt * ctx->diffusion[i]);
    }
    std::vector<float2> ff(ctx->ntype + 1);
    for (int i = 0; i <= ctx->ntype; ++i) ff[i] = make_float2((float)f1[i], (float)f2[i]);
    double *d1 = const_cast<double *>(p.fact1a), *d2 = const_cast<double *>(p.fact2a);
    float2 *d3 = const_cast<float2 *>(p.fact_f);
    int rc = upload(ctx, &d1, f1.data(), f1.size());
    if (!rc) rc = upload(ctx, &d2, f2.data(), f2.size());
    if (!rc) rc = upload(ctx, &d3, ff.data(), ff.size());
    p.fact1a = d1;
    p.fact2a = d2;
    p.fact_f = d3;
    if (rc) return rc;
  }
  return BROMOC_OK;
}

int bromoc_gpu_set_types(bromoc_ctx *ctx, const bromoc_types *t) {
  if (!ctx || !t || !t->nwtype || !t->cg || !t->diffusion)
    return set_err(ctx, BROMOC_E_ARG, "set_types: null");
  if (t->ntype < 1 || t->nttyp < 1 || t->nttyp > kMaxTypes || t->ndna < 0 ||
      t->nold < 0 || t->nold > t->ntype)
    return set_err(ctx, BROMOC_E_ARG, "set_types: bad sizes");
  for (int i = t->nold; i < t->ntype; ++i)
    if (t->nwtype[i] < 1 || t->nwtype[i] > t->nttyp)
      return set_err(ctx, BROMOC_E_ARG, "set_types: nwtype out of range");
  KP &p = ctx->kp;
  ctx->ntype = p.ntype = t->ntype;
  ctx->nold = p.nold = t->nold;
  ctx->nttyp = p.nttyp = t->nttyp;
  ctx->ndna = p.ndna = t->ndna;
  ctx->diffusion.assign(t->ntype + 1, 0.0);
  for (int i = 0; i < t->ntype; ++i) ctx->diffusion[i + 1] = t->diffusion[i];
  int rc = upload1(ctx, &p.nwtype, t->nwtype, t->ntype);
  if (!rc) rc = upload1(ctx, &p.cg, t->cg, t->ntype);
  if (!rc) rc = upload1(ctx, &p.diffusion, t->diffusion, t->ntype);
  if (!rc) {  // float-float charges of GRAND
    std::vector<float2> c(t->ntype), qc(t->ntype);
    for (int i = 0; i < t->ntype; ++i) {
      c[i] = ffsplit(t->cg[i]);
      qc[i] = ffsplit(p.celec * t->cg[i]);
    }
    rc = upload1(ctx, &p.cgff, c.data(), t->ntype);
    if (!rc) rc = upload1(ctx, &p.qcff, qc.data(), t->ntype);
  }
  if (rc) return rc;
  int *w = nullptr;
  if ((rc = dalloc(ctx, &w, t->nttyp + 1))) return rc;
  CU(cudaMemset(w, 0, (t->nttyp + 1) * sizeof(int)));
  p.warn = w;
  ctx->have_types = true;
  if (ctx->have_sys) return bromoc_gpu_set_system(ctx, &ctx->sys);
  return BROMOC_OK;
}

int bromoc_gpu_set_pairs(bromoc_ctx *ctx, const bromoc_pairs *q) {
  if (!ctx || !q) return set_err(ctx, BROMOC_E_ARG, "set_pairs: null");
  if (!ctx->have_types) return set_err(ctx, BROMOC_E_STATE, "set_pairs before set_types");
  const int ntc = q->ntc, nt = ctx->nttyp, ndna = ctx->ndna;
  const int nion = nt - ndna;
  if (ntc != (nt + ndna + 1) * nion / 2)
    return set_err(ctx, BROMOC_E_ARG, "set_pairs: ntc %d != (nttyp+ndna+1)*nion/2", ntc);
  if (!q->qchr || !q->qlj || !q->qsrpmf || !q->qefpot || !q->fct || !q->epp4 ||
      !q->sgp2 || !q->c0 || !q->c1 || !q->c2 || !q->c3 || !q->c4)
    return set_err(ctx, BROMOC_E_ARG, "set_pairs: null table");
  KP &p = ctx->kp;
  // packed pair index of every combined-type pair (nindex.f90:19-35)
  std::vector<int> pidx((size_t)nt * nt, -1);
  for (int a = 1; a <= nt; ++a)
    for (int b = 1; b <= nt; ++b) {
      if (a <= ndna && b <= ndna) continue;  // no site-site pair law
      int maxi, mini;
      if (a > b) {
        maxi = a - ndna;
        mini = b;
      } else {
        maxi = b - ndna;
        mini = a;
      }
      int is = mini > ndna ? maxi * (maxi - 1) / 2 + mini - ndna + ndna * nion
                           : (mini - 1) * nion + maxi;
      pidx[(size_t)(a - 1) * nt + (b - 1)] = is - 1;
    }
  const bool anyef = [&] {
    for (int k = 0; k < ntc; ++k)
      if (q->qefpot[k]) return true;
    return false;
  }();
  if (anyef && (!q->ep || !q->sc || !q->dm2 || !q->dmi || !q->nxi || q->cnt < 1 || q->res <= 0))
    return set_err(ctx, BROMOC_E_ARG, "set_pairs: effective-potential tables missing");
  // pieces per pair: up to the next pair's first piece
  std::vector<int> npieces(ntc, 0);
  for (int k = 0; k < ntc; ++k) {
    if (!q->qefpot[k]) continue;
    int next = q->cnt + 1;
    for (int m = 0; m < ntc; ++m)
      if (q->qefpot[m] && q->nxi[m] > q->nxi[k]) next = std::min(next, q->nxi[m]);
    npieces[k] = next - q->nxi[k];
    if (q->nxi[k] < 1 || npieces[k] < 1)
      return set_err(ctx, BROMOC_E_ARG, "set_pairs: bad nxi for pair %d", k + 1);
  }
  std::vector<PairParam> pp(ntc);
  std::vector<PairParamF> pf(ntc);
  std::vector<float4> ep32(anyef ? q->cnt : 1, make_float4(0, 0, 0, 0));
  for (int k = 0; k < ntc; ++k) {
    PairParam &a = pp[k];
    a = PairParam{};
    a.flags = (q->qchr[k] ? kChr : 0) | (q->qlj[k] ? kLj : 0) |
              (q->qsrpmf[k] ? kSrp : 0) | (q->qefpot[k] ? kEfp : 0);
    a.fct = q->fct[k];
    a.epp4 = q->epp4[k];
    a.sgp2 = q->sgp2[k];
    a.c0 = q->c0[k];
    a.c1 = q->c1[k];
    a.c2 = q->c2[k];
    a.c3 = q->c3[k];
    a.c4 = q->c4[k];
    if (q->qefpot[k]) {
      a.sc0 = q->sc[3 * k];
      a.sc1 = q->sc[3 * k + 1];
      a.sc2 = q->sc[3 * k + 2];
      a.dm2lo = q->dm2[2 * k];
      a.dm2hi = q->dm2[2 * k + 1];
      a.dmi = q->dmi[k];
      a.nxi = q->nxi[k] - 1;
      a.npieces = npieces[k];
      // local form about the bin start x_k = dmi + (k - nxi) res
      for (int m = 0; m < npieces[k]; ++m) {
        const int g = a.nxi + m;
        const double xk = a.dmi + m * q->res;
        const double p1 = q->ep[3 * g], p2 = q->ep[3 * g + 1], p3 = q->ep[3 * g + 2];
        ep32[g] = make_float4((float)(p1 + xk * (p2 + xk * p3)),
                              (float)(p2 + 2.0 * p3 * xk), (float)p3, (float)xk);
      }
    }
    PairParamF &f = pf[k];
    f.fct = (float)a.fct;
    f.epp4 = (float)a.epp4;
    f.sgp2 = (float)a.sgp2;
    f.c0 = (float)a.c0;
    f.c1 = (float)a.c1;
    f.c2 = (float)a.c2;
    f.c3 = (float)a.c3;
    f.c4 = (float)a.c4;
    f.sc0 = (float)a.sc0;
    f.sc1 = (float)a.sc1;
    f.sc2 = (float)a.sc2;
    f.dm2lo = (float)a.dm2lo;
    f.dm2hi = (float)a.dm2hi;
    f.dmi = (float)a.dmi;
    f.flags = a.flags | (a.npieces << 8);
    f.nxi = a.nxi;
  }
  p.rth = q->rth;
  p.srpx = q->srpx;
  p.srpk = q->srpk;
  p.srpy = q->srpy;
  p.res = q->res;
  p.ires = q->res > 0 ? 1.0 / q->res : 0.0;
  p.rthf = (float)p.rth;
  p.srpxf = (float)p.srpx;
  p.srpx2lo = (float)(p.srpx * p.srpx * (1.0 - kSrpWin));
  p.srpx2hi = (float)(p.srpx * p.srpx * (1.0 + kSrpWin));
  p.rthlo = (float)(p.rth * (1.0 - kSrpWin));
  p.rthhi = (float)(p.rth * (1.0 + kSrpWin));
  p.srpkf = (float)p.srpk;
  p.srpyf = (float)p.srpy;
  p.iresf = (float)p.ires;
  p.cnt = anyef ? q->cnt : 0;
  ctx->ntc = p.ntc = ntc;
  std::vector<float4> pk(4 * (size_t)ntc);
  auto bits = [](int v) {
    float f;
    std::memcpy(&f, &v, sizeof f);
    return f;
  };
  for (int k = 0; k < ntc; ++k) {
    const PairParamF &f = pf[k];
    pk[4 * k + 0] = make_float4(f.fct, f.epp4, f.sgp2, bits(f.flags));
    pk[4 * k + 1] = make_float4(f.c0, f.c1, f.c2, f.c3);
    pk[4 * k + 2] = make_float4(f.c4, f.sc0, f.sc1, f.sc2);
    pk[4 * k + 3] = make_float4(f.dm2lo, f.dm2hi, f.dmi, bits(f.nxi));
  }
  float4 *dpk = const_cast<float4 *>(p.ppk);
  if (int rc2 = upload(ctx, &dpk, pk.data(), pk.size())) return rc2;
  p.ppk = dpk;
  {  // float-float twins for GRAND
    std::vector<PairFF> pff(ntc);
    for (int k = 0; k < ntc; ++k) {
      const PairParam &a = pp[k];
      PairFF &f = pff[k];
      f.fct = ffsplit(a.fct);
      f.epp4 = ffsplit(a.epp4);
      f.sgp2 = ffsplit(a.sgp2);
      f.c0 = ffsplit(a.c0);
      f.c1 = ffsplit(a.c1);
      f.c2 = ffsplit(a.c2);
      f.c3pi = ffsplit(a.c3 * kPi);
      f.c4 = ffsplit(a.c4);
      f.sc0 = ffsplit(a.sc0);
      f.sc1 = ffsplit(a.sc1);
      f.sc2 = ffsplit(a.sc2);
      f.dm2lo = ffsplit(a.dm2lo);
      f.dm2hi = ffsplit(a.dm2hi);
      f.dmi = ffsplit(a.dmi);
      f.flags = a.flags;
      f.nxi = a.nxi;
      f.npieces = a.npieces;
      f.pad = 0;
    }
    std::vector<float2> eff(anyef ? 3 * (size_t)q->cnt : 3, make_float2(0.f, 0.f));
    if (anyef)
      for (size_t g = 0; g < 3 * (size_t)q->cnt; ++g) eff[g] = ffsplit(q->ep[g]);
    PairFF *dff = const_cast<PairFF *>(p.ppff);
    float2 *deff = const_cast<float2 *>(p.epff);
    int rc1 = upload(ctx, &dff, pff.data(), pff.size());
    if (!rc1) rc1 = upload(ctx, &deff, eff.data(), eff.size());
    p.ppff = dff;
    p.epff = deff;
    if (rc1) return rc1;
  }
  PairParam *dpp = const_cast<PairParam *>(p.pp);
  PairParamF *dpf = const_cast<PairParamF *>(p.ppf);
  int *dpi = const_cast<int *>(p.pidx);
  double *dep = const_cast<double *>(p.ep);
  float4 *de32 = const_cast<float4 *>(p.ep32);
  int rc = upload(ctx, &dpp, pp.data(), pp.size());
  if (!rc) rc = upload(ctx, &dpf, pf.data(), pf.size());
  if (!rc) rc = upload(ctx, &dpi, pidx.data(), pidx.size());
  if (!rc) rc = upload(ctx, &dep, anyef ? q->ep : nullptr, anyef ? 3 * (size_t)q->cnt : 3);
  if (!rc) rc = upload(ctx, &de32, ep32.data(), ep32.size());
  p.pp = dpp;
  p.ppf = dpf;
  p.pidx = dpi;
  p.ep = dep;
  p.ep32 = de32;
  if (rc) return rc;
  {  // dense ion-ion table of the FP32 pair kernel
    const int nion = nt - ndna;
    std::vector<float4> tab((size_t)nion * ipq_stride(nion),
                            make_float4(0.0f, 0.0f, 0.0f, -1.0f));
    bool ok = nion <= kIonTabTypes;
    for (int a = 0; a < nion && ok; ++a)
      for (int b = 0; b < nion; ++b) {
        const int is = pidx[(size_t)(a + ndna) * nt + (b + ndna)];
        const PairParamF &f = pf[is];
        if (f.flags & kEfp) ok = false;
        const int fl = f.flags & 15;
        // (fct, 6 epp4, sgp2, SRPMF cutoff on r^2 or -1): the LJ force takes
        // 6 epp4; the SRPMF test is one compare, against rth widened by the
        // window in which srp_branch decides in FP64
        tab[(size_t)a * ipq_stride(nion) + b] = make_float4(
            (fl & kChr) ? f.fct : 0.0f, (fl & kLj) ? 6.0f * f.epp4 : 0.0f,
            (fl & kLj) ? f.sgp2 : 0.0f, (fl & kSrp) ? p.rthhi : -1.0f);
      }
    float4 *dt = const_cast<float4 *>(p.ipq);
    if (!rc) rc = upload(ctx, &dt, tab.data(), std::max<size_t>(tab.size(), 1));
    p.ipq = dt;
    p.nion_t = nion;
    p.ipq_ok = ok ? 1 : 0;
    if (rc) return rc;
  }
  ctx->have_pairs = true;
  return BROMOC_OK;
}

int bromoc_gpu_set_sites(bromoc_ctx *ctx, const bromoc_sites *s) {
  if (!ctx || !s) return set_err(ctx, BROMOC_E_ARG, "set_sites: null");
  if (s->nsites < 0 || s->nsites > 1024)
    return set_err(ctx, BROMOC_E_ARG, "set_sites: nsites must be in [0, 1024]");
  KP &p = ctx->kp;
  p.nsites = s->nsites;
  clear_nucl(ctx);  // the term lists name sites of the previous set
  if (s->nsites == 0) return BROMOC_OK;
  if (!s->typtyp || !s->charge || !s->stfree)
    return set_err(ctx, BROMOC_E_ARG, "set_sites: null");
  for (int i = 0; i < s->nsites; ++i)
    if (s->typtyp[i] < 1 || s->typtyp[i] > ctx->ndna)
      return set_err(ctx, BROMOC_E_ARG, "set_sites: typtyp out of range");
  int *t = const_cast<int *>(p.typtyp);
  double *c = const_cast<double *>(p.sitecharge);
  uint8_t *f = const_cast<uint8_t *>(p.stfree);
  int rc = upload(ctx, &t, s->typtyp, s->nsites);
  if (!rc) rc = upload(ctx, &c, s->charge, s->nsites);
  if (!rc) rc = upload(ctx, &f, s->stfree, s->nsites);
  p.typtyp = t;
  p.sitecharge = c;
  p.stfree = f;
  if (!rc && ctx->precision == BROMOC_FP32) {  // partials of the FP32 ion-site tiles
    for (void *a : {(void *)p.isp_ion, (void *)p.isp_site, (void *)p.isp_dids,
                    (void *)p.isp_seed})
      dfree(ctx, a);
    p.isp_ion = p.isp_site = p.isp_dids = p.isp_seed = nullptr;
    p.isp_tcap = 0;
    const size_t S = (s->nsites + kIsSiteTile - 1) / kIsSiteTile, cap = p.cap;
    const int T = (int)((cap + 31) / 32);
    rc = dalloc(ctx, &p.isp_ion, S * 3 * cap);
    if (!rc) rc = dalloc(ctx, &p.isp_dids, S * 6 * cap);
    if (!rc) rc = dalloc(ctx, &p.isp_seed, 5 * cap);
    if (!rc) rc = dalloc(ctx, &p.isp_site, (size_t)T * 3 * s->nsites);
    if (!rc) p.isp_tcap = T;
  }
  ctx->site_map.clear();
  if (!rc && s->phiv_map) {
    if (p.qphiv && p.qnmcden) {
      int nmaps = ctx->phiv_nmaps;
      for (int i = 0; i < s->nsites; ++i)
        if (s->phiv_map[i] < 0 || s->phiv_map[i] >= nmaps)
          return set_err(ctx, BROMOC_E_ARG, "set_sites: phiv_map out of range");
    }
    ctx->site_map.assign(s->phiv_map, s->phiv_map + s->nsites);
    int *m = const_cast<int *>(p.site_map);
    rc = upload(ctx, &m, s->phiv_map, s->nsites);
    p.site_map = m;
  } else if (p.qphiv && p.qnmcden) {
    return set_err(ctx, BROMOC_E_ARG, "set_sites: nmcden needs per-site maps");
  }
  return rc;
}

int bromoc_gpu_set_mmij(bromoc_ctx *ctx, const bromoc_mmij *q) {
  if (!ctx) return BROMOC_E_ARG;
  CU(cudaStreamSynchronize(ctx->stream));
  clear_mmij(ctx);
  if (!q) return BROMOC_OK;
  KP &p = ctx->kp;
  MmijDev &m = p.mm;
  std::vector<int3> lst;
  std::vector<double> bn;
  if (q->shape == BROMOC_BOX) {
    if (q->xnpol < 1 || q->ynpol < 1 || q->znpol < 1 || q->xnpol > 64 || q->ynpol > 64 ||
        q->znpol > 64 || !q->lstpx || !q->lstpy || !q->lstpz || !q->mmij ||
        !(q->rbxmax - q->rbxmin > 0.0) || !(q->rbymax - q->rbymin > 0.0) ||
        !(q->rbzmax - q->rbzmin > 0.0))
      return set_err(ctx, BROMOC_E_ARG, "set_mmij: RECTBOX orders (1..64), region or matrix");
    const int nt = q->xnpol * q->ynpol * q->znpol;
    m.rect = 1;
    m.nx = q->xnpol;
    m.ny = q->ynpol;
    m.nz = q->znpol;
    m.ntpol = nt;
    // shell_simul.f90:2792-2802, rect_norm.f90
    m.xscal = 2.0 / (q->rbxmax - q->rbxmin);
    m.yscal = 2.0 / (q->rbymax - q->rbymin);
    m.zscal = 2.0 / (q->rbzmax - q->rbzmin);
    m.xmax = 1.0 / m.xscal;
    m.ymax = 1.0 / m.yscal;
    m.zmax = 1.0 / m.zscal;
    m.rfscal = q->rfscal;
    const double ilxyz = m.xscal * m.yscal * m.zscal * 0.125;
    for (int n = 0; n < nt; ++n) {
      const int a = q->lstpx[n], b = q->lstpy[n], c = q->lstpz[n];
      if (a < 0 || a >= m.nx || b < 0 || b >= m.ny || c < 0 || c >= m.nz)
        return set_err(ctx, BROMOC_E_ARG, "set_mmij: basis order out of range");
      lst.push_back(make_int3(a, b, c));
      bn.push_back(std::sqrt((2.0 * a + 1.0) * (2.0 * b + 1.0) * (2.0 * c + 1.0) * ilxyz));
    }
  } else if (q->shape == BROMOC_SPHERE) {
    if (q->nmpol < 1 || q->nmpol > 25 || !(q->srdist > 0.0) || !q->mmij)
      return set_err(ctx, BROMOC_E_ARG, "set_mmij: SPHERE nmpol (1..25), srdist or matrix");
    m.rect = 0;
    m.nmpol = q->nmpol;
    m.ntpol = q->nmpol * q->nmpol;
    m.srdist2 = q->srdist * q->srdist;
    // sphe_svpol.f90, sphe_norm.f90 (factori.f90)
    auto fact = [](int n) {
      double f = 1.0;
      for (int i = 2; i <= n; ++i) f = f * i;
      return f;
    };
    const double sr2 = q->srdist * q->srdist, itwopi = 1.0 / (2.0 * 3.14159265358979323846);
    double rpart = sr2 * q->srdist, lpart = 1.5 * itwopi;
    const double ipi = 0.5 * itwopi;
    lst.push_back(make_int3(0, 0, 0));
    bn.push_back(std::sqrt(lpart / rpart));
    for (int l = 1; l < q->nmpol; ++l) {
      lpart = (2.0 * l + 1.0) * (2.0 * l + 3.0) * ipi;
      rpart = rpart * sr2;
      lst.push_back(make_int3(l, 0, 0));
      bn.push_back(std::sqrt(lpart / rpart));
      lpart = (2.0 * l + 1.0) * (2.0 * l + 3.0) * itwopi;
      for (int mm = 1; mm <= l; ++mm) {
        const double v = std::sqrt(lpart * fact(l - mm) / (rpart * fact(l + mm)));
        lst.push_back(make_int3(l, mm, 0));
        bn.push_back(v);
        lst.push_back(make_int3(l, -mm, 0));
        bn.push_back(v);
      }
    }
  } else {
    return set_err(ctx, BROMOC_E_ARG, "set_mmij: shape must be BROMOC_BOX or BROMOC_SPHERE");
  }
  const int nt = m.ntpol;
  std::vector<double> mat(q->mmij, q->mmij + (size_t)nt * nt);
  for (int i = 0; i < nt; ++i)  // readmmij.f90: the lower triangle from the upper
    for (int j = 0; j < i; ++j) mat[(size_t)i * nt + j] = mat[(size_t)j * nt + i];
  m.tabw = mmij_table_width(m.rect, m.nx, m.ny, m.nz, m.nmpol);
  const size_t cap = p.cap;
  const int nch = std::max(1, (int)((cap + 1 + 255) / 256));
  int3 *dl = nullptr;
  double *db = nullptr, *dm = nullptr;
  int rc = upload(ctx, &dl, lst.data(), lst.size());
  if (!rc) rc = upload(ctx, &db, bn.data(), bn.size());
  if (!rc) rc = upload(ctx, &dm, mat.data(), mat.size());
  if (!rc) rc = dalloc(ctx, &m.tab, (cap + 1) * (size_t)m.tabw);
  if (!rc) rc = dalloc(ctx, &m.in, cap + 1);
  if (!rc) rc = dalloc(ctx, &m.ist, cap + 2);
  if (!rc) rc = dalloc(ctx, &m.coefp, (size_t)nch * nt);
  if (!rc) rc = dalloc(ctx, &m.coef, (size_t)nt);
  if (!rc) rc = dalloc(ctx, &m.coef2, (size_t)nt);
  if (!rc) rc = dalloc(ctx, &m.mq, (size_t)nt);
  if (!rc) rc = dalloc(ctx, &m.rowe, (size_t)nt);
  m.lst = dl;
  m.bnorm = db;
  m.m = dm;
  if (!rc) rc = cudaMemset(m.in, 0, cap + 1) == cudaSuccess ? 0 : BROMOC_E_CUDA;
  if (rc) {
    clear_mmij(ctx);
    return rc ? rc : set_err(ctx, BROMOC_E_CUDA, "set_mmij: device memory");
  }
  m.on = 1;
  return BROMOC_OK;
}

int bromoc_gpu_set_nucleotides(bromoc_ctx *ctx, const bromoc_nucleotides *q) {
  if (!ctx) return BROMOC_E_ARG;
  CU(cudaStreamSynchronize(ctx->stream));
  clear_nucl(ctx);
  if (!q) return BROMOC_OK;
  const int ns = ctx->kp.nsites;
  if (ns <= 0) return set_err(ctx, BROMOC_E_STATE, "set_nucleotides: set_sites first");
  // term list in kind order: bond, angle, torsion, stack, base pair,
  // excluded volume, qq, solvent, APFOR
  const int cnt[kNucKinds] = {q->nbond, q->nangle, q->ndihe, q->nstack, q->nbp,
                              q->nex,   q->nqq,    q->nsolv, q->afn};
  const int per[kNucKinds] = {2, 3, 4, 2, 2, 2, 2, 2, 1};
  const int32_t *lst[kNucKinds] = {q->sitebond, q->siteangle, q->sitedihe, q->sitestack,
                                   q->sitebp,   q->siteex,    q->siteqq,   q->siteslv,
                                   q->sn};
  const double *val[kNucKinds] = {q->distbond, q->valangle, q->valdihe, q->sgstack, q->sgbp,
                                  q->sgex,     nullptr,     nullptr,    nullptr};
  NucDev &n = ctx->kp.nuc;
  std::vector<int4> site;
  std::vector<double> par;
  int total = 0;
  for (int k = 0; k < kNucKinds; ++k) {
    if (cnt[k] < 0 || cnt[k] > (1 << 24))
      return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: count out of range");
    if (cnt[k] > 0 && (!lst[k] || (k < 6 && !val[k])))
      return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: null list");
    n.off[k] = total;
    total += cnt[k];
  }
  n.off[kNucKinds] = total;
  if (q->nbp > 0 && !q->bpgc) return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: null bpgc");
  if (q->afn > 0 && !q->af) return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: null af");
  site.reserve(total);
  par.reserve(total);
  std::vector<std::vector<int>> ent(ns);  // per site: 4t+m, ascending t
  for (int k = 0; k < kNucKinds; ++k)
    for (int i = 0; i < cnt[k]; ++i) {
      int v[4] = {-1, -1, -1, -1};
      for (int m = 0; m < per[k]; ++m) {
        const int sj = lst[k][per[k] * i + m];
        if (sj < 1 || sj > ns)
          return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: site %d out of [1, %d]", sj, ns);
        v[m] = sj - 1;
        ent[sj - 1].push_back(4 * (int)site.size() + m);
      }
      if (k == 4) v[2] = q->bpgc[i] ? 1 : 0;
      site.push_back(make_int4(v[0], v[1], v[2], v[3]));
      par.push_back(val[k] ? val[k][i] : 0.0);
    }
  std::vector<int> start(ns + 1, 0), flat;
  for (int j = 0; j < ns; ++j) {
    start[j] = (int)flat.size();
    flat.insert(flat.end(), ent[j].begin(), ent[j].end());
  }
  start[ns] = (int)flat.size();
  const int ctn = q->ctn;
  if (ctn < 0 || (ctn > 0 && (!q->csn || !q->kx || !q->ky || !q->kz || !q->contrx ||
                              !q->contry || !q->contrz)))
    return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: CONTRANS lists");
  std::vector<double> ck(3 * (size_t)std::max(ctn, 1), 0.0), cc(3 * (size_t)(ctn + 1), 0.0);
  for (int i = 0; i < ctn; ++i) {
    if (q->csn[i] < 0 || q->csn[i] > ns)
      return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: csn out of [0, nsites]");
    ck[3 * i] = q->kx[i];
    ck[3 * i + 1] = q->ky[i];
    ck[3 * i + 2] = q->kz[i];
  }
  for (int i = 0; i <= ctn && ctn > 0; ++i) {
    cc[3 * i] = q->contrx[i];
    cc[3 * i + 1] = q->contry[i];
    cc[3 * i + 2] = q->contrz[i];
  }
  if (q->qunsplit && (q->nsites1st < 1 || q->nsites1st >= ns))
    return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: nsites1st out of [1, nsites)");
  if (q->qdeby && !(q->kappa > 0.0))
    return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: Debye length must be positive");
  if (q->qdeby < 0 || q->qdeby > 2)
    return set_err(ctx, BROMOC_E_ARG, "set_nucleotides: qdeby must be 0, 1 or 2");
  int4 *dsite = nullptr;
  double *dpar = nullptr, *daf = nullptr, *dck = nullptr, *dcc = nullptr;
  int *dstart = nullptr, *dflat = nullptr, *dcsn = nullptr;
  int rc = upload(ctx, &dsite, site.data(), site.size());
  if (!rc) rc = upload(ctx, &dpar, par.data(), par.size());
  if (!rc) rc = upload(ctx, &daf, q->af, 3 * (size_t)q->afn);
  if (!rc) rc = upload(ctx, &dstart, start.data(), start.size());
  if (!rc) rc = upload(ctx, &dflat, flat.data(), flat.size());
  if (!rc) rc = upload(ctx, &dcsn, q->csn, (size_t)ctn);
  if (!rc) rc = upload(ctx, &dck, ck.data(), ck.size());
  if (!rc) rc = upload(ctx, &dcc, cc.data(), cc.size());
  if (!rc) rc = dalloc(ctx, &n.te, (size_t)total);
  if (!rc) rc = dalloc(ctx, &n.tf, (size_t)total * 12);
  if (!rc) rc = dalloc(ctx, &n.cf, 8);
  n.site = dsite;
  n.par = dpar;
  n.af = daf;
  n.csr_start = dstart;
  n.csr_ent = dflat;
  n.csn = dcsn;
  n.ck = dck;
  n.cc = dcc;
  if (rc) {
    clear_nucl(ctx);
    return rc;
  }
  n.nterm = total;
  n.epsnuc = q->epsnuc;
  n.scalepairing = q->scalepairing;
  n.fctn = q->fctn;
  n.kappa = q->kappa;
  n.ikappa = q->qdeby ? 1.0 / q->kappa : 0.0;
  n.epsolv = q->epsolv;
  n.qdeby = q->qdeby;
  n.qsolv = q->qsolv != 0;
  n.ctn = ctn;
  n.qunsplit = q->qunsplit != 0;
  n.nsites1st = q->nsites1st;
  for (int a = 0; a < 3; ++a) {
    n.qnotr[a] = q->qnotr[a] != 0;
    n.notr[a] = q->notr[a];
  }
  ctx->nuc_on = true;
  return BROMOC_OK;
}

int bromoc_gpu_set_phix(bromoc_ctx *ctx, const bromoc_grid *g, const float *phix) {
  if (!ctx || !grid_ok(g) || !phix) return set_err(ctx, BROMOC_E_ARG, "set_phix: bad grid");
  KP &p = ctx->kp;
  p.g1 = make_grid(*g);
  float *d = const_cast<float *>(p.phix);
  int rc = upload(ctx, &d, phix, (size_t)g->nclx * g->ncly * g->nclz);
  p.phix = d;
  if (!rc) p.qphix = 1;
  return rc;
}

int bromoc_gpu_set_phiv(bromoc_ctx *ctx, const bromoc_grid *g, const int8_t *phiv,
                        const bromoc_phiv_opts *o) {
  if (!ctx || !grid_ok(g) || !phiv || !o || o->nmaps < 1)
    return set_err(ctx, BROMOC_E_ARG, "set_phiv: bad arguments");
  if (o->nmcden && !o->map_of_type)
    return set_err(ctx, BROMOC_E_ARG, "set_phiv: nmcden needs map_of_type");
  KP &p = ctx->kp;
  {
    const Grid3 gg = make_grid(*g);  // vzmin/vzmax inside the map (shell_simul:2759,2763)
    if (o->vzmax > gg.zbcen + gg.tranz || o->vzmin < gg.zbcen - gg.tranz)
      return set_err(ctx, BROMOC_E_ARG, "set_phiv: vzmin/vzmax outside the map");
    if (o->nmcden && p.nsites > 0) {
      if (ctx->site_map.empty())
        return set_err(ctx, BROMOC_E_ARG, "set_phiv: nmcden needs per-site maps");
      for (int m : ctx->site_map)
        if (m < 0 || m >= o->nmaps)
          return set_err(ctx, BROMOC_E_ARG, "set_phiv: site map out of range");
    }
  }
  p.g2 = make_grid(*g);
  int8_t *d = const_cast<int8_t *>(p.phiv);
  int rc = upload(ctx, &d, phiv, (size_t)o->nmaps * g->nclx * g->ncly * g->nclz);
  p.phiv = d;
  if (rc) return rc;
  p.qtrln = o->trilinear != 0;
  p.qnmcden = o->nmcden != 0;
  p.svdw = o->svdw;
  p.vzmin = o->vzmin;
  p.vzmax = o->vzmax;
  p.thold8 = o->thold8;
  p.thold27 = o->thold27;
  if (o->map_of_type) {
    for (int i = ctx->nold; i < ctx->ntype; ++i)
      if (o->map_of_type[i] < 0 || o->map_of_type[i] >= o->nmaps)
        return set_err(ctx, BROMOC_E_ARG, "set_phiv: map_of_type out of range");
    if ((rc = upload1(ctx, &p.phiv_map_of_type, o->map_of_type, ctx->ntype))) return rc;
  }
  p.qsvdw = o->scal != nullptr;
  if (o->scal && (rc = upload1(ctx, &p.scal, o->scal, ctx->nttyp))) return rc;
  {  // repulsion scale per combined type for the FP32 kernels (phiv_select)
    std::vector<float> es(ctx->nttyp + 1, (float)o->svdw);
    if (!o->nmcden && o->scal)
      for (int t = 1; t <= ctx->nttyp; ++t) es[t] = (float)(o->svdw * o->scal[t - 1]);
    float *d = const_cast<float *>(p.esvdw_f);
    rc = upload(ctx, &d, es.data(), es.size());
    p.esvdw_f = d;
    if (rc) return rc;
    std::vector<float2> ef(ctx->nttyp + 1, ffsplit(o->svdw));  // float-float, for GRAND
    if (!o->nmcden && o->scal)
      for (int t = 1; t <= ctx->nttyp; ++t) ef[t] = ffsplit(o->svdw * o->scal[t - 1]);
    float2 *df = const_cast<float2 *>(p.esvff);
    rc = upload(ctx, &df, ef.data(), ef.size());
    p.esvff = df;
    if (rc) return rc;
  }
  ctx->phiv_nmaps = o->nmaps;
  p.qphiv = 1;
  return BROMOC_OK;
}

int bromoc_gpu_set_rfpar(bromoc_ctx *ctx, const bromoc_grid *g, int32_t nmaps,
                         const float *gsrfen, const float *greff, double reffac,
                         const int32_t *map_of_type) {
  if (!ctx || !grid_ok(g) || !gsrfen || !greff || nmaps < 1 || reffac < 0)
    return set_err(ctx, BROMOC_E_ARG, "set_rfpar: bad arguments");
  KP &p = ctx->kp;
  p.g3 = make_grid(*g);
  const size_t n = (size_t)nmaps * g->nclx * g->ncly * g->nclz;
  float *a = const_cast<float *>(p.gsrfen), *b = const_cast<float *>(p.greff);
  int rc = upload(ctx, &a, gsrfen, n);
  if (!rc) rc = upload(ctx, &b, greff, n);
  p.gsrfen = a;
  p.greff = b;
  if (rc) return rc;
  p.sqrfac = std::sqrt(reffac);  // shell_simul.f90:2860
  p.qrfpsin = map_of_type == nullptr;
  if (map_of_type) {
    for (int i = ctx->nold; i < ctx->ntype; ++i)
      if (map_of_type[i] < 0 || map_of_type[i] >= nmaps)
        return set_err(ctx, BROMOC_E_ARG, "set_rfpar: map_of_type out of range");
    if ((rc = upload1(ctx, &p.rfpar_map_of_type, map_of_type, ctx->ntype))) return rc;
  }
  p.qrfpar = 1;
  return BROMOC_OK;
}

int bromoc_gpu_set_membrane(bromoc_ctx *ctx, const bromoc_membrane *m) {
  if (!ctx || !m || !m->ampl1 || !m->p1 || !m->ampl2 || !m->p2 || !m->rcylinder)
    return set_err(ctx, BROMOC_E_ARG, "set_membrane: null");
  if (!ctx->have_types) return set_err(ctx, BROMOC_E_STATE, "set_membrane before set_types");
  KP &p = ctx->kp;
  const int n = ctx->nttyp;
  std::vector<double> p1a(n), p1b(n), p2a(n), p2b(n);
  for (int i = 0; i < n; ++i) {
    p1a[i] = m->p1[2 * i];
    p1b[i] = m->p1[2 * i + 1];
    p2a[i] = m->p2[2 * i];
    p2b[i] = m->p2[2 * i + 1];
  }
  int rc = upload1(ctx, &p.ampl1, m->ampl1, n);
  if (!rc) rc = upload1(ctx, &p.ampl2, m->ampl2, n);
  if (!rc) rc = upload1(ctx, &p.rcyl, m->rcylinder, n);
  if (!rc) rc = upload1(ctx, &p.p1a, p1a.data(), n, 1.0);
  if (!rc) rc = upload1(ctx, &p.p1b, p1b.data(), n, 1.0);
  if (!rc) rc = upload1(ctx, &p.p2a, p2a.data(), n, 1.0);
  if (!rc) rc = upload1(ctx, &p.p2b, p2b.data(), n, 1.0);
  if (rc) return rc;
  p.qpore = m->qpore;
  p.voltage = m->voltage;
  p.afact = m->afact;
  p.ikappa = m->ikappa;
  p.ceps = m->ceps;
  p.zmemb1 = m->zmemb1;
  p.zmemb2 = m->zmemb2;
  p.qmemb = 1;
  return BROMOC_OK;
}

int bromoc_gpu_set_diffusion(bromoc_ctx *ctx, const bromoc_diffusion *d) {
  if (!ctx || !d) return set_err(ctx, BROMOC_E_ARG, "set_diffusion: null");
  if (!ctx->have_types) return set_err(ctx, BROMOC_E_STATE, "set_diffusion before set_types");
  KP &p = ctx->kp;
  int rc = upload1(ctx, &p.ampl3, d->ampl3, ctx->ntype);
  if (!rc) rc = upload1(ctx, &p.p3, d->p3, ctx->ntype, 1.0);
  if (rc) return rc;
  p.plength2 = d->plength2;
  p.pcenter = d->pcenter;
  p.nspline = d->nspline;
  if (d->nspline > 0) {
    if (!d->xs || !d->ys || !d->b || !d->c || !d->d)
      return set_err(ctx, BROMOC_E_ARG, "set_diffusion: spline arrays missing");
    rc = upload1(ctx, &p.xs, d->xs, d->nspline);
    if (!rc) rc = upload1(ctx, &p.ys, d->ys, d->nspline);
    if (!rc) rc = upload1(ctx, &p.sb, d->b, d->nspline);
    if (!rc) rc = upload1(ctx, &p.scc, d->c, d->nspline);
    if (!rc) rc = upload1(ctx, &p.sd, d->d, d->nspline);
    if (rc) return rc;
  }
  p.diff0 = d->diff0;
  p.ibeta = d->ibeta;
  p.diffcutoff = d->diffcutoff;
  p.qproxdiff = d->diffcutoff > 0.0;
  p.fact0n1 = d->fact0n1;
  p.fact0n2 = d->fact0n2;
  p.qdnafree = d->qdnafree;
  return BROMOC_OK;
}

int bromoc_gpu_set_countions(bromoc_ctx *ctx, int32_t cntpts, const double *zcont) {
  if (!ctx || cntpts < 0 || (cntpts > 0 && !zcont))
    return set_err(ctx, BROMOC_E_ARG, "set_countions: bad arguments");
  if (!ctx->have_types) return set_err(ctx, BROMOC_E_STATE, "set_countions before set_types");
  KP &p = ctx->kp;
  ctx->cntpts = p.cntpts = cntpts;
  if (cntpts == 0) return BROMOC_OK;
  double *z = const_cast<double *>(p.zcont);
  int rc = upload(ctx, &z, zcont, cntpts);
  p.zcont = z;
  std::vector<float2> zf(cntpts);
  for (int j = 0; j < cntpts; ++j) split_ff(zcont[j], zf[j].x, zf[j].y);
  float2 *zd = const_cast<float2 *>(p.zcont_ff);
  if (!rc) rc = upload(ctx, &zd, zf.data(), zf.size());
  p.zcont_ff = zd;
  const size_t n = (size_t)(ctx->ntype - ctx->nold) * cntpts;
  if (!rc) rc = upload<int>(ctx, &p.nforward, nullptr, n);
  if (!rc) rc = upload<int>(ctx, &p.nbackward, nullptr, n);
  if (rc) return rc;
  CU(cudaMemset(p.nforward, 0, n * sizeof(int)));
  CU(cudaMemset(p.nbackward, 0, n * sizeof(int)));
  return BROMOC_OK;
}

int bromoc_gpu_set_buffers(bromoc_ctx *ctx, const bromoc_buffers *b) {
  if (!ctx || !b) return set_err(ctx, BROMOC_E_ARG, "set_buffers: null");
  if (b->nbuffer < 0 || b->nbuffer > kMaxBuffers)
    return set_err(ctx, BROMOC_E_ARG, "set_buffers: nbuffer must be in [0, %d]", kMaxBuffers);
  KP &p = ctx->kp;
  const int n = b->nbuffer;
  ctx->nbuffer = p.nbuffer = n;
  if (n == 0) return BROMOC_OK;
  if (!b->ibfftyp || !b->avnum || !b->mu || !b->kb || !b->lzmin || !b->lzmax ||
      !b->qbufferbias || !b->nat || !b->ntotat)
    return set_err(ctx, BROMOC_E_ARG, "set_buffers: null array");
  if (!ctx->have_types) return set_err(ctx, BROMOC_E_STATE, "set_buffers before set_types");
  for (int i = 0; i < n; ++i) {
    if (b->ibfftyp[i] <= ctx->nold || b->ibfftyp[i] > ctx->ntype)
      return set_err(ctx, BROMOC_E_ARG, "set_buffers: buffer %d ion type %d out of range",
                     i + 1, b->ibfftyp[i]);
    if (b->nat[i] < 0 || b->nat[i] > p.cap)
      return set_err(ctx, BROMOC_E_ARG, "set_buffers: nat(%d) out of range", i + 1);
  }
  int rc = upload1(ctx, &p.ibfftyp, b->ibfftyp, n);
  if (!rc) rc = upload1(ctx, &p.avnum, b->avnum, n);
  if (!rc) rc = upload1(ctx, &p.mu, b->mu, n);
  if (!rc) rc = upload1(ctx, &p.kbb, b->kb, n);
  if (!rc) {  // float-float (avnum, mu, kb) per buffer for GRAND's acceptance, 1-based
    std::vector<float2> v(3 * (size_t)(n + 1), make_float2(0.f, 0.f));
    for (int i = 0; i < n; ++i) {
      v[3 * (i + 1)] = ffsplit(b->avnum[i]);
      v[3 * (i + 1) + 1] = ffsplit(b->mu[i]);
      v[3 * (i + 1) + 2] = ffsplit(b->kb[i]);
    }
    float2 *d = const_cast<float2 *>(p.bufff);
    rc = upload(ctx, &d, v.data(), v.size());
    p.bufff = d;
  }
  if (!rc) rc = upload1(ctx, &p.lzmin, b->lzmin, n);
  if (!rc) rc = upload1(ctx, &p.lzmax, b->lzmax, n);
  if (!rc) rc = upload1(ctx, &p.rmin, b->rmin, n);
  if (!rc) rc = upload1(ctx, &p.rmax, b->rmax, n);
  if (!rc) rc = upload1(ctx, &p.qbufferbias, b->qbufferbias, n);
  if (!rc) rc = upload<int>(ctx, &p.prob, nullptr, (size_t)n * (p.cap + 1));
  if (rc) return rc;
  CU(cudaMemset(p.prob, 0, (size_t)n * (p.cap + 1) * sizeof(int)));
  DevState h{};
  CU(cudaMemcpy(&h, p.st, sizeof h, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) {
    h.nat[i] = b->nat[i];
    h.ntotat[i] = b->ntotat[i];
    h.ninsert[i] = 0;
    h.nremove[i] = 0;
  }
  CU(cudaMemcpy(p.st, &h, sizeof h, cudaMemcpyHostToDevice));
  return BROMOC_OK;
}

}  // extern "C"

namespace {

// Host arrays -> device.  Stream-ordered after earlier work; with wait the
// call returns once the copies are done (the caller may reuse its buffers).
int upload_particles(bromoc_ctx *ctx, int32_t ntot, int32_t nsites, int32_t nfix,
                     const double *x, const double *y, const double *z, const int32_t *typei,
                     const int32_t *ibuffer, bool wait) {
  if (!ctx || !x || !y || !z || !typei) return set_err(ctx, BROMOC_E_ARG, "set_particles: null");
  KP &p = ctx->kp;
  if (ntot < 0 || ntot > p.cap)
    return set_err(ctx, BROMOC_E_CAPACITY, "set_particles: ntot %d exceeds capacity %d", ntot, p.cap);
  if (nsites != p.nsites)
    return set_err(ctx, BROMOC_E_STATE, "set_particles: nsites %d differs from set_sites (%d)",
                   nsites, p.nsites);
  if (nfix < 0 || nsites + nfix > ntot)
    return set_err(ctx, BROMOC_E_ARG, "set_particles: bad nfix");
  if (!ctx->have_types) return set_err(ctx, BROMOC_E_STATE, "set_particles before set_types");
  for (int i = nsites; i < ntot; ++i) {
    const int t = typei[i] < 0 ? -typei[i] : typei[i];
    if (t <= ctx->nold || t > ctx->ntype)
      return set_err(ctx, BROMOC_E_ARG, "set_particles: typei(%d) = %d is not an ion type",
                     i + 1, typei[i]);
  }
  // the count goes up from its own pinned word: a read-back still pending on
  // the stream targets word 0 and would overwrite it before the upload
  if (wait) CU(cudaStreamSynchronize(ctx->stream));
  p.nfix = nfix;
  const size_t n = (size_t)std::max(ntot, 1);
  CU(cudaMemcpyAsync(p.x, x, ntot * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(p.y, y, ntot * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(p.z, z, ntot * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CU(cudaMemcpyAsync(p.typei, typei, ntot * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if (ibuffer)
    CU(cudaMemcpyAsync(p.ibuffer, ibuffer, ntot * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  else
    CU(cudaMemsetAsync(p.ibuffer, 0, n * sizeof(int), ctx->stream));
  ctx->h_ntot[4] = ntot;
  CU(cudaMemcpyAsync(&p.st->ntot, ctx->h_ntot + 4, sizeof(int), cudaMemcpyHostToDevice,
                     ctx->stream));
  if (wait) CU(cudaStreamSynchronize(ctx->stream));
  ctx->ntot_known = ntot;
  ctx->attempts_at_known = ctx->attempts_total;
  ctx->rb_pending = false;
  ctx->have_forces = false;
  ctx->ff_fresh = false;
  ctx->dbl_fresh = true;
  return BROMOC_OK;
}

// Device -> host arrays with one wait: the count, the error word and, for
// each array, the entries up to the count's host-side upper bound (the
// buffers are capacity-sized) travel together.  *err receives the word.
int download_particles(bromoc_ctx *ctx, int32_t *ntot, double *x, double *y, double *z,
                       int32_t *typei, int32_t *ibuffer, int *err) {
  int rc = ensure_dbl(ctx);
  if (rc) return rc;
  KP &p = ctx->kp;
  const int ub = ntot_ub(ctx);
  CU(cudaMemcpyAsync(ctx->h_ntot, &p.st->ntot, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                     ctx->stream));
  int lo = 0, hi = ub;
  for (int pass = 0; pass < 2; ++pass) {
    const size_t m = (size_t)(hi - lo);
    if (m) {
      if (x) CU(cudaMemcpyAsync(x + lo, p.x + lo, m * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      if (y) CU(cudaMemcpyAsync(y + lo, p.y + lo, m * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      if (z) CU(cudaMemcpyAsync(z + lo, p.z + lo, m * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      if (typei)
        CU(cudaMemcpyAsync(typei + lo, p.typei + lo, m * sizeof(int), cudaMemcpyDeviceToHost,
                           ctx->stream));
      if (ibuffer)
        CU(cudaMemcpyAsync(ibuffer + lo, p.ibuffer + lo, m * sizeof(int), cudaMemcpyDeviceToHost,
                           ctx->stream));
    }
    CU(cudaStreamSynchronize(ctx->stream));
    const int n = ctx->h_ntot[0];
    if (n <= hi) break;
    lo = hi;  // the bound is exact by construction; this pass never runs
    hi = std::min(n, p.cap);
  }
  ctx->ntot_known = ctx->h_ntot[0];
  ctx->attempts_at_known = ctx->attempts_total;
  ctx->rb_pending = false;
  if (ntot) *ntot = ctx->ntot_known;
  if (err) *err = ctx->h_ntot[1];
  return BROMOC_OK;
}

}  // namespace

extern "C" {

int bromoc_gpu_set_particles(bromoc_ctx *ctx, int32_t ntot, int32_t nsites,
                             int32_t nfix, const double *x, const double *y,
                             const double *z, const int32_t *typei,
                             const int32_t *ibuffer) {
  return upload_particles(ctx, ntot, nsites, nfix, x, y, z, typei, ibuffer, true);
}

int bromoc_gpu_get_particles(bromoc_ctx *ctx, int32_t *ntot, double *x, double *y,
                             double *z, int32_t *typei, int32_t *ibuffer) {
  if (!ctx) return BROMOC_E_ARG;
  int rc = ensure_dbl(ctx);
  if (!rc) rc = sync_ntot(ctx);
  if (rc) return rc;
  const int n = ctx->ntot_known;
  KP &p = ctx->kp;
  if (ntot) *ntot = n;
  if (x) CU(cudaMemcpyAsync(x, p.x, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (y) CU(cudaMemcpyAsync(y, p.y, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (z) CU(cudaMemcpyAsync(z, p.z, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (typei) CU(cudaMemcpyAsync(typei, p.typei, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (ibuffer)
    CU(cudaMemcpyAsync(ibuffer, p.ibuffer, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return BROMOC_OK;
}

int bromoc_gpu_energy(bromoc_ctx *ctx, uint32_t terms, int32_t qforces, double *fx,
                      double *fy, double *fz, double *eterms, int32_t *warn) {
  if (!ctx) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  KP &p = ctx->kp;
  EnergyPlan plan{};
  AssembleFlags fl{};
  if ((rc = plan_energy(ctx, terms, true, plan, fl))) return rc;
  if ((rc = ensure_ff(ctx))) return rc;
  CU(cudaMemsetAsync(p.warn, 0, (ctx->nttyp + 1) * sizeof(int), ctx->stream));
  ctx->launches += launch_energy(p, plan, terms, qforces, ctx->stream);
  launch_assemble(p, plan.ntot_ub, fl, 0, 0, 0, 0, ctx->stream);
  ctx->launches += plan.ntot_ub > 0;
  CU(cudaGetLastError());
  if ((rc = sync_ntot(ctx))) return rc;
  const int n = ctx->ntot_known;
  if (eterms)
    CU(cudaMemcpyAsync(eterms, p.eterms, kNTerms * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
  if (qforces) {
    if (fx) CU(cudaMemcpyAsync(fx, p.fx, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (fy) CU(cudaMemcpyAsync(fy, p.fy, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (fz) CU(cudaMemcpyAsync(fz, p.fz, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (warn)
    CU(cudaMemcpyAsync(warn, p.warn + 1, ctx->nttyp * sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->have_forces = qforces != 0;
  return check_device_err(ctx);
}

int bromoc_gpu_interact(bromoc_ctx *ctx, uint32_t terms, double xj, double yj, double zj,
                        int32_t jtype, int32_t j, double *dener) {
  if (!ctx || !dener) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if ((rc = ensure_dbl(ctx))) return rc;
  if ((rc = sync_ntot(ctx))) return rc;
  KP &p = ctx->kp;
  const int ntot = ctx->ntot_known;
  if (j < 1 || j > ntot + 1) return set_err(ctx, BROMOC_E_ARG, "interact: j out of range");
  if (j == ntot + 1 && ntot + 1 > p.cap)
    return set_err(ctx, BROMOC_E_CAPACITY, "interact: no room for the trial slot");
  const bool beion = j > p.nsites;
  if (beion && (jtype <= ctx->nold || jtype > ctx->ntype))
    return set_err(ctx, BROMOC_E_ARG, "interact: jtype %d is not an ion type", jtype);
  Trial t{};
  t.valid = 1;
  t.insert = j == ntot + 1;
  t.itype = jtype;
  t.j = j;
  t.x = xj;
  t.y = yj;
  t.z = zj;
  CU(cudaMemcpyAsync(p.trial, &t, sizeof t, cudaMemcpyHostToDevice, ctx->stream));
  launch_interact(p, ntot, terms, 1, ctx->d_dener, ctx->stream);
  ctx->launches += 3;
  if (!beion && ctx->nuc_on) {  // the site's bonded/Go terms (interact.f90:211-334)
    launch_nucl_interact(p, terms, j - 1, ctx->d_dener, ctx->stream);
    ++ctx->launches;
  }
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(dener, ctx->d_dener, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return check_device_err(ctx);
}

int bromoc_gpu_metropolis(bromoc_ctx *ctx, uint32_t terms, int32_t nmcm, double mcmax,
                          uint64_t seed, uint64_t cycle, int32_t *naccept,
                          double *dener_sum) {
  if (!ctx || nmcm < 0 || !(mcmax > 0.0)) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if ((rc = ensure_dbl(ctx))) return rc;
  if ((rc = sync_ntot(ctx))) return rc;
  KP &p = ctx->kp;
  if (p.nfix > 0)
    return set_err(ctx, BROMOC_E_STATE,
                   "metropolis: systems with fixed ions are not supported (move.f90 draws "
                   "the ion over ntot - nsites slots)");
  const int ntot = ctx->ntot_known;
  if (ntot - p.nsites < 1) return set_err(ctx, BROMOC_E_STATE, "metropolis: no mobile ion");
  if (!ctx->mc && (rc = dalloc(ctx, &ctx->mc, 1))) return rc;
  CU(cudaMemsetAsync(ctx->mc, 0, sizeof(McState), ctx->stream));
  ctx->launches += launch_metropolis(p, ntot, terms, nmcm, mcmax, seed, cycle, ctx->mc,
                                     ctx->stream);
  CU(cudaGetLastError());
  McState h{};
  CU(cudaMemcpyAsync(&h, ctx->mc, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  if (naccept) *naccept = h.naccept;
  if (dener_sum) *dener_sum = h.dener;
  if (ctx->precision == BROMOC_FP32) ctx->ff_fresh = false;  // the FP64 arrays moved
  return check_device_err(ctx);
}

int bromoc_gpu_dynamics(bromoc_ctx *ctx, int32_t variant, uint64_t seed, uint64_t step) {
  if (!ctx) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (!ctx->have_forces)
    return set_err(ctx, BROMOC_E_STATE, "dynamics: call energy with forces first");
  if (variant < 0 || variant > 3) return set_err(ctx, BROMOC_E_ARG, "dynamics: bad variant");
  KP &p = ctx->kp;
  if (variant == BROMOC_DYN2 && p.nspline < 2)
    return set_err(ctx, BROMOC_E_STATE, "dynamics2 needs a PROFILE spline");
  AssembleFlags fl{};  // the force is fx,fy,fz as the last energy call left it
  fl.fp32_noise = ctx->precision == BROMOC_FP32;
  fl.fp32_partials = ctx->precision == BROMOC_FP32;
  fl.use_total = 1;
  if ((rc = ensure_ff(ctx))) return rc;
  launch_assemble(p, ntot_ub(ctx), fl, 1, variant, seed, step, ctx->stream);
  ctx->launches += 1;
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->have_forces = false;
  if (ctx->precision == BROMOC_FP32) ctx->dbl_fresh = false;
  return BROMOC_OK;
}

int bromoc_gpu_bd_steps(bromoc_ctx *ctx, uint32_t terms, int32_t variant, int32_t nsteps,
                        uint64_t seed, uint64_t step0, double *eterms) {
  if (!ctx) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (variant < 0 || variant > 3) return set_err(ctx, BROMOC_E_ARG, "bd_steps: bad variant");
  if (nsteps < 0) return set_err(ctx, BROMOC_E_ARG, "bd_steps: nsteps < 0");
  KP &p = ctx->kp;
  if (variant == BROMOC_DYN2 && p.nspline < 2)
    return set_err(ctx, BROMOC_E_STATE, "dynamics2 needs a PROFILE spline");
  if (variant == BROMOC_DYN3 && !p.qproxdiff)
    return set_err(ctx, BROMOC_E_STATE, "dynamics3 needs PROXDIFF (diffcutoff > 0)");
  EnergyPlan plan{};
  AssembleFlags fl{};
  if ((rc = ensure_ff(ctx))) return rc;
  if (ctx->precision == BROMOC_FP32 && nsteps > 0) ctx->dbl_fresh = false;
  int k = 0;
  // FP32 Newton-3 systems without sites: the steps whose energy is not
  // wanted run as one cooperative launch (loop.cu) with the forces, moves
  // and summation order of the per-kernel steps below.
  const int nloop = eterms ? nsteps - 1 : nsteps;
  if (ctx->fused_bd && ctx->precision == BROMOC_FP32 && nloop > 0) {
    if ((rc = plan_energy(ctx, terms, false, plan, fl, false))) return rc;
    if (bd_loop_supported(p, fl) && !plan.mmij) {
      KTimer *tl = next_timer(ctx, BROMOC_K_LOOP);
      if (tl) cudaEventRecord(tl->a, ctx->stream);
      CU(launch_bd_loop(p, fl, plan.ntot_ub, terms, variant, seed, step0, nloop, 1,
                        ctx->stream));
      if (tl) cudaEventRecord(tl->b, ctx->stream);
      ctx->launches += 1;
      k = nloop;
    }
  }
  for (; k < nsteps; ++k) {
    const bool last = k + 1 == nsteps;
    if ((rc = plan_energy(ctx, terms, last && eterms, plan, fl))) return rc;
    ctx->launches += launch_energy(p, plan, terms, 1, ctx->stream);
    KTimer *ta = plan.ntot_ub > 0 ? next_timer(ctx, BROMOC_K_ASSEMBLE) : nullptr;
    if (ta) cudaEventRecord(ta->a, ctx->stream);
    launch_assemble(p, plan.ntot_ub, fl, 1, variant, seed, step0 + k, ctx->stream);
    if (plan.nuc) ctx->launches += launch_notrans(p, plan.fp32, ctx->stream);  // simul1.f90:380
    if (ta) cudaEventRecord(ta->b, ctx->stream);
    ctx->launches += plan.ntot_ub > 0;
  }
  CU(cudaGetLastError());
  ctx->have_forces = false;
  if (eterms && nsteps > 0) {
    CU(cudaMemcpyAsync(eterms, p.eterms, kNTerms * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return check_device_err(ctx);
  }
  return BROMOC_OK;
}

int bromoc_gpu_bd_steps_host(bromoc_ctx *ctx, uint32_t terms, int32_t variant, int32_t nsteps,
                             uint64_t seed, uint64_t step0, int32_t ntot, int32_t nsites,
                             int32_t nfix, double *x, double *y, double *z,
                             const int32_t *typei, double *eterms) {
  if (!ctx || !x || !y || !z || !typei) return set_err(ctx, BROMOC_E_ARG, "bd_steps_host: null");
  // the host arrays are read and rewritten in stream order: one wait, at the end
  int rc = upload_particles(ctx, ntot, nsites, nfix, x, y, z, typei, nullptr, false);
  if (!rc) rc = bromoc_gpu_bd_steps(ctx, terms, variant, nsteps, seed, step0, eterms);
  if (!rc) rc = ensure_dbl(ctx);
  if (!rc) {
    KP &p = ctx->kp;
    CU(cudaMemcpyAsync(x, p.x, ntot * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(y, p.y, ntot * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(z, p.z, ntot * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaMemcpyAsync(ctx->h_ntot + 1, &p.st->err, sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
  }
  cudaStreamSynchronize(ctx->stream);  // also on an error: no copy outlives the call
  if (!rc) rc = device_err_result(ctx, ctx->h_ntot[1]);
  return rc;
}

int bromoc_gpu_grand(bromoc_ctx *ctx, uint32_t terms, int32_t ngcmc, uint64_t seed,
                     uint64_t cycle, double *dener_sum) {
  if (!ctx) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  KP &p = ctx->kp;
  if (ngcmc < 0 || cycle < 1) return set_err(ctx, BROMOC_E_ARG, "grand: bad ngcmc or cycle");
  if (p.nbuffer < 1) return set_err(ctx, BROMOC_E_STATE, "grand: no buffers");
  // with the MMIJ reaction field the attempts run one after another
  // through INTERACT (launch_grand_seq), on the FP64 arrays
  const bool seq = p.mm.on && (terms & BROMOC_M_MMIJ);
  // FP32 mode: GRAND works on the float-float records (the current
  // positions while BD runs), FP64 mode on the FP64 arrays
  const bool ff = ctx->precision == BROMOC_FP32 && !seq;
  if ((rc = ff ? ensure_ff(ctx) : ensure_dbl(ctx))) return rc;
  if (ngcmc > 0) {
    if (ff)
      ctx->dbl_fresh = false;
    else
      ctx->ff_fresh = false;
  }
  // the kernel starts its energy sum at zero; without a launch, zero it here
  if (ngcmc == 0) CU(cudaMemsetAsync(&p.st->dener_sum, 0, sizeof(double), ctx->stream));
  {  // float-float constants of the GRAND kernel's ΔE
    FFC &f = p.ffc;
    const Grid3 *gs[3] = {&p.g1, &p.g2, &p.g3};
    for (int m = 0; m < 3; ++m) {
      const Grid3 &g = *gs[m];
      const double tr[3] = {g.tranx, g.trany, g.tranz}, bc[3] = {g.xbcen, g.ybcen, g.zbcen};
      const int ncl[3] = {g.nclx, g.ncly, g.nclz};
      for (int a = 0; a < 3; ++a) {
        f.g[m].ub[a] = ffsplit(bc[a] + tr[a]);
        f.g[m].lb[a] = ffsplit(bc[a] - tr[a]);
        f.g[m].o[a] = ffsplit(tr[a] - bc[a]);
        f.g[m].ncl[a] = ncl[a];
      }
      f.g[m].dcel = ffsplit(g.dcel);
      f.g[m].idcel = ffsplit(g.idcel);
    }
    f.sqrfac = ffsplit(p.sqrfac);
    f.thold8 = ffsplit(p.thold8);
    f.thold27 = ffsplit(p.thold27);
    f.vzmin = ffsplit(p.vzmin);
    f.vzmax = ffsplit(p.vzmax);
    f.rth = ffsplit(p.rth);
    f.srpx = ffsplit(p.srpx);
    f.srpk = ffsplit(p.srpk);
    f.srpy = ffsplit(p.srpy);
    f.ires = ffsplit(p.ires);
    f.ikbt = ffsplit(p.ikbt);
    const double L[3] = {p.lx, p.ly, p.lz};
    for (int a = 0; a < 3; ++a) {
      f.L[a] = ffsplit(L[a]);
      f.iL[a] = L[a] > 0.0 ? (float)(1.0 / L[a]) : 0.0f;
    }
    f.rc2 = ffsplit(p.rc2);
  }
  if (ngcmc > 0) {
    KTimer *tg = next_timer(ctx, BROMOC_K_GRAND);
    if (tg) cudaEventRecord(tg->a, ctx->stream);
    if (seq) {
      ctx->launches += launch_grand_seq(p, ntot_ub(ctx), terms, seed, cycle, ngcmc,
                                        ctx->d_dener, ctx->stream);
    } else {
      CU(launch_grand(p, ntot_ub(ctx), ctx->ipart_slots, terms, seed, cycle, ngcmc, ff ? 1 : 0,
                      ctx->stream));
      ctx->launches += 1;
    }
    if (tg) cudaEventRecord(tg->b, ctx->stream);
    ctx->attempts_total += ngcmc;
  }
  CU(cudaGetLastError());
  if (!ctx->rb_pending) {  // refresh the ntot bound without blocking
    CU(cudaMemcpyAsync(ctx->h_ntot, &p.st->ntot, sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CU(cudaEventRecord(ctx->ev_ntot, ctx->stream));
    ctx->rb_pending = true;
    ctx->rb_attempts = ctx->attempts_total;
  }
  ctx->have_forces = false;
  if (dener_sum) {
    CU(cudaMemcpyAsync(ctx->h_ntot + 2, &p.st->dener_sum, sizeof(double),
                       cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    std::memcpy(dener_sum, ctx->h_ntot + 2, sizeof(double));
    return check_device_err(ctx);
  }
  return BROMOC_OK;
}

int bromoc_gpu_get_buffers(bromoc_ctx *ctx, int32_t *nat, int32_t *ninsert, int32_t *nremove,
                           int32_t *prob) {
  if (!ctx) return BROMOC_E_ARG;
  KP &p = ctx->kp;
  DevState h{};
  CU(cudaStreamSynchronize(ctx->stream));
  CU(cudaMemcpy(&h, p.st, sizeof h, cudaMemcpyDeviceToHost));
  for (int i = 0; i < ctx->nbuffer; ++i) {
    if (nat) nat[i] = h.nat[i];
    if (ninsert) ninsert[i] = h.ninsert[i];
    if (nremove) nremove[i] = h.nremove[i];
  }
  if (prob && ctx->nbuffer > 0)
    CU(cudaMemcpy(prob, p.prob, (size_t)ctx->nbuffer * (p.cap + 1) * sizeof(int),
                  cudaMemcpyDeviceToHost));
  return BROMOC_OK;
}

int bromoc_gpu_get_countions(bromoc_ctx *ctx, int32_t *nf, int32_t *nb) {
  if (!ctx) return BROMOC_E_ARG;
  KP &p = ctx->kp;
  const size_t n = (size_t)(ctx->ntype - ctx->nold) * ctx->cntpts;
  CU(cudaStreamSynchronize(ctx->stream));
  if (n == 0) return BROMOC_OK;
  if (nf) CU(cudaMemcpy(nf, p.nforward, n * sizeof(int), cudaMemcpyDeviceToHost));
  if (nb) CU(cudaMemcpy(nb, p.nbackward, n * sizeof(int), cudaMemcpyDeviceToHost));
  return BROMOC_OK;
}

int64_t bromoc_gpu_launch_count(const bromoc_ctx *ctx) {
  return ctx ? (int64_t)ctx->launches : -1;
}

int bromoc_gpu_live_count_async(bromoc_ctx *ctx, int32_t *dst) {
  if (!ctx || !dst) return BROMOC_E_ARG;
  CU(cudaMemcpyAsync(dst, &ctx->kp.st->ntot, sizeof(int32_t), cudaMemcpyDeviceToHost,
                     ctx->stream));
  return BROMOC_OK;
}

int bromoc_gpu_set_periodic(bromoc_ctx *ctx, int32_t on, double rcut) {
  if (!ctx) return BROMOC_E_ARG;
  if (on && (!ctx->have_sys || ctx->sys.shape != BROMOC_BOX))
    return set_err(ctx, BROMOC_E_STATE, "set_periodic: needs set_system with a box");
  if (on && !(rcut > 0.0)) return set_err(ctx, BROMOC_E_ARG, "set_periodic: rcut must be > 0");
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->kp.periodic = on != 0;
  ctx->kp.rc2 = on ? rcut * rcut : 0.0;
  return BROMOC_OK;
}

int bromoc_gpu_set_fused_bd(bromoc_ctx *ctx, int32_t on) {
  if (!ctx) return BROMOC_E_ARG;
  ctx->fused_bd = on != 0;
  return BROMOC_OK;
}

int bromoc_gpu_kernel_timing(bromoc_ctx *ctx, int32_t on) {
  if (!ctx) return BROMOC_E_ARG;
  CU(cudaStreamSynchronize(ctx->stream));
  ctx->timing = on != 0;
  for (int k = 0; k < BROMOC_K_NKINDS; ++k) ctx->tused[k] = 0;
  return BROMOC_OK;
}

int bromoc_gpu_kernel_time(bromoc_ctx *ctx, int32_t which, double *total_ms,
                           int64_t *launches) {
  if (!ctx || which < 0 || which >= BROMOC_K_NKINDS || !total_ms || !launches)
    return set_err(ctx, BROMOC_E_ARG, "kernel_time: bad arguments");
  CU(cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  for (int i = 0; i < ctx->tused[which]; ++i) {
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, ctx->tpool[which][i].a, ctx->tpool[which][i].b));
    sum += ms;
  }
  *total_ms = sum;
  *launches = ctx->tused[which];
  return BROMOC_OK;
}

int bromoc_gpu_simul_cycles_host(bromoc_ctx *ctx, uint32_t terms, int32_t variant,
                                 int32_t ncycle, int32_t ngcmc, int32_t nbd, uint64_t seed,
                                 uint64_t cycle0, int32_t *ntot, int32_t nsites, int32_t nfix,
                                 double *x, double *y, double *z, int32_t *typei,
                                 int32_t *ibuffer, double *eterms) {
  if (!ctx || !ntot || !x || !y || !z || !typei || !ibuffer)
    return set_err(ctx, BROMOC_E_ARG, "simul_cycles_host: null");
  if (ncycle < 0 || ngcmc < 0 || nbd < 0 || cycle0 < 1)
    return set_err(ctx, BROMOC_E_ARG, "simul_cycles_host: bad counts");
  // the host arrays are read and rewritten in stream order: one wait, at the end
  int rc = upload_particles(ctx, *ntot, nsites, nfix, x, y, z, typei, ibuffer, false);
  for (int c = 0; !rc && c < ncycle; ++c) {
    const uint64_t cyc = cycle0 + c;
    if (ngcmc > 0) rc = bromoc_gpu_grand(ctx, terms, ngcmc, seed, cyc, nullptr);
    if (!rc && nbd > 0)
      rc = bromoc_gpu_bd_steps(ctx, terms, variant, nbd, seed, (cyc - 1) * nbd,
                               c + 1 == ncycle ? eterms : nullptr);
    if (!rc) rc = bromoc_gpu_count(ctx);  // simul1.f90:462 (nothing without buffers)
    if (!rc && ctx->prof_on) rc = bromoc_gpu_accum_profiles(ctx);  // simul1.f90:476-509
  }
  int e = 0;
  if (!rc) rc = download_particles(ctx, ntot, x, y, z, typei, ibuffer, &e);
  if (!rc) rc = device_err_result(ctx, e);
  if (rc) cudaStreamSynchronize(ctx->stream);  // no copy outlives the call
  return rc;
}

int bromoc_gpu_count(bromoc_ctx *ctx) {
  if (!ctx) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if (ctx->kp.nbuffer < 1) return BROMOC_OK;
  const bool ff = ctx->precision == BROMOC_FP32;
  if ((rc = ff ? ensure_ff(ctx) : ensure_dbl(ctx))) return rc;
  ctx->launches += launch_count(ctx->kp, ff, ntot_ub(ctx), ctx->stream);
  CU(cudaGetLastError());
  return BROMOC_OK;
}

int bromoc_gpu_get_ntotat(bromoc_ctx *ctx, int32_t *ntotat) {
  if (!ctx || !ntotat) return BROMOC_E_ARG;
  const int nb = ctx->kp.nbuffer;
  if (nb > 0) {
    CU(cudaMemcpyAsync(ntotat, ctx->kp.st->ntotat, nb * sizeof(int), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
  }
  return BROMOC_OK;
}

int bromoc_gpu_set_profiles(bromoc_ctx *ctx, int32_t qrho, int32_t qrdna, int32_t qgr,
                            int32_t igr, double dr, int32_t npoints) {
  if (!ctx) return BROMOC_E_ARG;
  if (!ctx->have_sys || !ctx->have_types)
    return set_err(ctx, BROMOC_E_STATE, "set_profiles: set_system and set_types first");
  if (npoints < 1 || (qgr && (!(dr > 0.0) || igr < 1 || igr > ctx->kp.cap)))
    return set_err(ctx, BROMOC_E_ARG, "set_profiles: npoints, dr or igr out of range");
  CU(cudaStreamSynchronize(ctx->stream));
  ProfArgs &a = ctx->prof;
  for (void *q : {(void *)a.rho_n, (void *)a.rdna_n, (void *)a.gr_n, (void *)a.irmax})
    dfree(ctx, q);
  a = ProfArgs{};
  ctx->prof_on = false;
  if (!qrho && !qrdna && !qgr) return BROMOC_OK;
  const KP &p = ctx->kp;
  // simul1.f90:179-188
  a.zmini = p.lz2m;
  a.idelz = 2.0;
  a.nzmax = std::min((int)(p.lz * a.idelz), (int)npoints);
  a.rho = qrho != 0;
  a.rdna = qrdna != 0 && p.nsites > 0;
  a.gr = qgr != 0;
  a.igr = igr - 1;
  a.dr = dr;
  a.npoints = npoints;
  const int nion_t = ctx->ntype - ctx->nold;
  int rc = dalloc(ctx, &a.rho_n, (size_t)std::max(nion_t, 1) * std::max(a.nzmax, 1));
  if (!rc) rc = dalloc(ctx, &a.rdna_n, (size_t)std::max(ctx->ndna, 1) * std::max(a.nzmax, 1));
  if (!rc) rc = dalloc(ctx, &a.gr_n, (size_t)std::max(nion_t, 1) * npoints);
  if (!rc) rc = dalloc(ctx, &a.irmax, 1);
  if (rc) return rc;
  CU(cudaMemset(a.rho_n, 0, (size_t)std::max(nion_t, 1) * std::max(a.nzmax, 1) * 8));
  CU(cudaMemset(a.rdna_n, 0, (size_t)std::max(ctx->ndna, 1) * std::max(a.nzmax, 1) * 8));
  CU(cudaMemset(a.gr_n, 0, (size_t)std::max(nion_t, 1) * npoints * 8));
  CU(cudaMemset(a.irmax, 0, sizeof(int)));
  ctx->prof_on = true;
  return BROMOC_OK;
}

int bromoc_gpu_accum_profiles(bromoc_ctx *ctx) {
  if (!ctx) return BROMOC_E_ARG;
  if (!ctx->prof_on) return set_err(ctx, BROMOC_E_STATE, "accum_profiles: set_profiles first");
  int rc = check_ready(ctx);
  if (rc) return rc;
  launch_profiles(ctx->kp, ctx->precision == BROMOC_FP32, ntot_ub(ctx), ctx->prof, ctx->stream);
  ++ctx->launches;
  CU(cudaGetLastError());
  return BROMOC_OK;
}

int bromoc_gpu_get_profiles(bromoc_ctx *ctx, double *rho, double *rdna, double *gr,
                            int32_t *nzmax, int32_t *irmax) {
  if (!ctx) return BROMOC_E_ARG;
  if (!ctx->prof_on) return set_err(ctx, BROMOC_E_STATE, "get_profiles: set_profiles first");
  const ProfArgs &a = ctx->prof;
  const int nion_t = ctx->ntype - ctx->nold;
  auto fetch = [&](const unsigned long long *src, size_t n, double *dst) -> int {
    if (!dst || !src || n == 0) return BROMOC_OK;
    std::vector<unsigned long long> h(n);
    CU(cudaMemcpyAsync(h.data(), src, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    for (size_t k = 0; k < n; ++k) dst[k] = (double)h[k];
    return BROMOC_OK;
  };
  int rc = fetch(a.rho_n, a.rho ? (size_t)nion_t * a.nzmax : 0, rho);
  if (!rc) rc = fetch(a.rdna_n, a.rdna ? (size_t)ctx->ndna * a.nzmax : 0, rdna);
  if (!rc) rc = fetch(a.gr_n, a.gr ? (size_t)nion_t * a.npoints : 0, gr);
  if (rc) return rc;
  if (nzmax) *nzmax = a.nzmax;
  if (irmax) {
    CU(cudaMemcpyAsync(irmax, a.irmax, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
  }
  return BROMOC_OK;
}

int bromoc_gpu_traj_header(int32_t nframe, int32_t nttyp, const char *atnam, void *buf,
                           int64_t cap, int64_t *nbytes) {
  if (nttyp < 0 || (nttyp > 0 && !atnam) || !nbytes) return BROMOC_E_ARG;
  const int64_t n = 12 + 12 + 8 + 4 * (int64_t)nttyp;
  *nbytes = n;
  if (!buf) return BROMOC_OK;  // size query
  if (cap < n) return BROMOC_E_ARG;
  uint8_t *b = (uint8_t *)buf;
  const int32_t w[6] = {4, nframe, 4, 4, nttyp, 4};
  std::memcpy(b, w, 24);
  const int32_t L = 4 * nttyp;
  std::memcpy(b + 24, &L, 4);
  if (nttyp) std::memcpy(b + 28, atnam, 4 * (size_t)nttyp);
  std::memcpy(b + 28 + 4 * (size_t)nttyp, &L, 4);
  return BROMOC_OK;
}

int bromoc_gpu_traj_frame(bromoc_ctx *ctx, double runtime, void *buf, int64_t cap,
                          int64_t *nbytes) {
  if (!ctx || !nbytes) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if ((rc = sync_ntot(ctx))) return rc;
  const int n = ctx->ntot_known;
  const long long nb = 60 + 16 * (long long)n;
  *nbytes = nb;
  if (!buf) return BROMOC_OK;  // size query
  if (cap < nb) return set_err(ctx, BROMOC_E_ARG, "traj_frame: buffer holds %lld of %lld bytes",
                               (long long)cap, nb);
  if (nb > ctx->traj_cap) {
    dfree(ctx, ctx->traj_w);
    ctx->traj_w = nullptr;
    ctx->traj_cap = 0;
    if ((rc = dalloc(ctx, &ctx->traj_w, (size_t)(nb / 4)))) return rc;
    ctx->traj_cap = nb;
  }
  launch_traj_pack(ctx->kp, ctx->precision == BROMOC_FP32, n, runtime, ctx->traj_w,
                   ctx->stream);
  ++ctx->launches;
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(buf, ctx->traj_w, (size_t)nb, cudaMemcpyDeviceToHost, ctx->stream));
  CU(cudaStreamSynchronize(ctx->stream));
  return check_device_err(ctx);
}

int bromoc_gpu_get_dids(bromoc_ctx *ctx, double *dids) {
  if (!ctx || !dids) return BROMOC_E_ARG;
  int rc = check_ready(ctx);
  if (rc) return rc;
  if ((rc = sync_ntot(ctx))) return rc;
  CU(cudaMemcpy(dids, ctx->kp.dids, 5 * (size_t)ctx->ntot_known * sizeof(double),
                cudaMemcpyDeviceToHost));
  return BROMOC_OK;
}

}  // extern "C"
