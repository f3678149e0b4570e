// Reaction field of the MMIJ basis (gsbpmod), FP64 in both modes.
//
// ENERGY (rect_rf1.f90, sphe_rf1.f90):
//   k_mmij_tab    one thread per particle: in-region flag and the basis
//                 tables of its position (RECTBOX: Legendre values and
//                 slopes per axis; SPHERE: r^l, cos/sin(m phi), P_l^m and
//                 dP_l^m/d cos(theta)), into its row of MmijDev::tab;
//   k_mmij_coef   one thread per basis function and ion chunk: the chunk's
//                 sum of q_i b(r_i) into coefp (no atomics);
//   k_mmij_sum    coef = the chunk sums in chunk order; the SPHERE forces'
//                 10/sin(theta) of the last ion in the sphere;
//   k_mmij_mq     one warp per row: mq = M coef (x rfscal for RECTBOX),
//                 lanes over the row, a fixed shuffle tree;
//   k_mmij_energy one block: egsbpb = celec sum coef mq / 2 into an energy
//                 slot;
//   k_mmij_force  one thread per ion in the region: -q celec sum_k grad b_k
//                 mq_k, added to the field forces (ffield / ffield_f).
// INTERACT (rect_rf0.f90, sphe_rf0.f90): the same tables with particle j at
// the trial position (an extra row for an insertion trial), coef2 = coef -
// q_j b(r_j), then per row k the terms of E(coef) - E(coef2) over l >= k
// (k_mmij_qform) and their sum (k_mmij_iafinal), added to INTERACT's
// result.  Particles outside the region, and j that is not a mobile ion,
// contribute nothing.
#include <algorithm>

#include "launch.h"
#include "physics.cuh"

namespace bgpu {

constexpr int kMmThreads = 128;
constexpr int kMmChunk = 256;  // ions per partial-sum chunk

template <bool F32>
__device__ __forceinline__ void mm_pos(const KP &p, int i, double r[3]) {
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

// Sphere table layout within a row of tab
struct SpheLayout {
  int lmax, mc, w;  // w: (l, m) row width of P and dP
  __host__ __device__ int ar() const { return 0; }
  __host__ __device__ int ac() const { return lmax + 1; }
  __host__ __device__ int as() const { return lmax + 1 + mc + 1; }
  __host__ __device__ int ap() const { return lmax + 1 + 2 * (mc + 1); }
  __host__ __device__ int adp() const { return ap() + (lmax + 2) * w; }
  __host__ __device__ int ang() const { return adp() + (lmax + 2) * w; }  // st, ct, cp, sp
  __host__ __device__ int width() const { return ang() + 4; }
};

__host__ __device__ inline SpheLayout sphe_layout(int nmpol) {
  SpheLayout L;
  L.lmax = nmpol - 1;
  L.mc = L.lmax > 3 ? L.lmax : 3;
  L.w = L.lmax + 2;
  return L;
}

// The tables of one position into t; false when outside the region.
// istnum is 10 for ENERGY (sphe_rf1.f90:46) and 1 for INTERACT.
__device__ bool mm_tables(const KP &p, const double r[3], double istnum, double *t,
                          double &ist) {
  const MmijDev &m = p.mm;
  ist = 0.0;
  if (m.rect) {
    if (!(r[0] >= -m.xmax && r[0] <= m.xmax && r[1] >= -m.ymax && r[1] <= m.ymax &&
          r[2] >= -m.zmax && r[2] <= m.zmax))
      return false;
    const double sc[3] = {m.xscal, m.yscal, m.zscal};
    const int np[3] = {m.nx, m.ny, m.nz};
    int off = 0;
    for (int a = 0; a < 3; ++a) {
      const double xs = sc[a] * r[a];
      double *v = t + off, *d = t + off + np[a];
      // rect_rf1.f90:33-55 and :88-118 (values, then slopes, scaled)
      double v0 = 1.0, v1 = xs, v2 = 0.5 * (3.0 * xs * xs - 1.0);
      double d0 = 0.0, d1 = 1.0, d2 = 3.0 * xs;
      v[0] = v0;
      d[0] = d0 * sc[a];
      if (np[a] > 1) {
        v[1] = v1;
        d[1] = d1 * sc[a];
      }
      if (np[a] > 2) {
        v[2] = v2;
        d[2] = d2 * sc[a];
      }
      double vm2 = v1, vm1 = v2, dm1 = d2;
      for (int n = 3; n <= np[a] - 1; ++n) {
        const double vn = ((2.0 * n - 1) * xs * vm1 - (n - 1.0) * vm2) / n;
        const double dn = xs * dm1 + n * vm1;
        v[n] = vn;
        d[n] = dn * sc[a];
        vm2 = vm1;
        vm1 = vn;
        dm1 = dn;
      }
      off += 2 * np[a];
    }
    return true;
  }
  const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  if (!(r2 <= m.srdist2)) return false;
  const SpheLayout L = sphe_layout(m.nmpol);
  const double rr = sqrt(r2), ir = 1.0 / rr;
  double ct = r[2] * ir;
  double st = sqrt(1.0 - ct * ct);
  ist = istnum / st;
  double cp = r[0] * ir * ist, sp = r[1] * ir * ist;
  if (r2 < 1e-3) {  // rsmall: at the origin
    ct = st = cp = sp = 0.0;
  } else if (r[0] > -1e-3 && r[0] < 1e-3 && r[1] > -1e-3 && r[1] < 1e-3) {  // z axis
    ct = r[2] < 0.0 ? -1.0 : 1.0;
    cp = sp = 0.0;
  } else if (r[2] > -1e-3 && r[2] < 1e-3) {  // xy plane
    ct = 0.0;
    cp = r[0] * ir;
    sp = r[1] * ir;
  }
  double *ar = t + L.ar(), *ac = t + L.ac(), *as = t + L.as();
  double *ap = t + L.ap(), *adp = t + L.adp();
  ar[0] = 1.0;  // rpowerl2
  for (int i = 1; i <= L.lmax; ++i) ar[i] = ar[i - 1] * rr;
  ac[0] = 1.0;  // cosmphi2, sinmphi2
  ac[1] = cp;
  ac[2] = 2.0 * cp * cp - 1.0;
  ac[3] = (2.0 * ac[2] - 1.0) * cp;
  as[0] = 0.0;
  as[1] = sp;
  as[2] = 2.0 * cp * sp;
  as[3] = 2.0 * cp * as[2] - sp;
  for (int i = 4; i <= L.lmax; ++i) {
    ac[i] = 2.0 * cp * ac[i - 1] - ac[i - 2];
    as[i] = 2.0 * cp * as[i - 1] - as[i - 2];
  }
  const int W = L.w, lmax = L.lmax, mmax = L.lmax;
  for (int k = 0; k < (lmax + 2) * W; ++k) ap[k] = 0.0;  // P_l^m = 0 for m > l
  const double xc = ct;
  ap[0] = 1.0;  // alpol2
  const double somx2 = sqrt((1.0 - xc) * (1.0 + xc));
  double fact = 1.0;
  for (int mm = 1; mm <= mmax; ++mm) {
    ap[mm * W + mm] = ap[(mm - 1) * W + mm - 1] * fact * somx2;
    fact = fact + 2.0;
  }
  for (int mm = 0; mm <= mmax; ++mm) ap[(mm + 1) * W + mm] = xc * (2 * mm + 1) * ap[mm * W + mm];
  for (int l = 2; l <= lmax; ++l)
    for (int mm = 0; mm <= l - 2; ++mm)
      ap[l * W + mm] =
          (xc * (2.0 * l - 1) * ap[(l - 1) * W + mm] - (l + mm - 1) * ap[(l - 2) * W + mm]) /
          (l - mm);
  if (xc == 1.0 || xc == -1.0) {  // dalpol2
    for (int l = 0; l <= lmax; ++l) {
      double v = 0.0;
      if (xc == 1.0) v = l * (l + 1.0) * 0.5;
      if (xc == -1.0) v = ((l + 1) % 2 ? -1.0 : 1.0) * l * (l + 1.0) * 0.5;
      adp[l * W] = v;
      for (int mm = 1; mm <= mmax; ++mm) adp[l * W + mm] = 0.0;
    }
  } else {
    for (int l = 0; l <= lmax; ++l)
      for (int mm = 0; mm <= mmax; ++mm) {
        const double f = 1.0 / sqrt(1.0 - xc * xc);
        adp[l * W + mm] = f * (ap[l * W + mm + 1] - f * mm * xc * ap[l * W + mm]);
      }
  }
  double *ang = t + L.ang();
  ang[0] = st;
  ang[1] = ct;
  ang[2] = cp;
  ang[3] = sp;
  return true;
}

// basis function k (without its norm) of a table row
__device__ __forceinline__ double mm_value(const MmijDev &m, int k, const double *t) {
  const int3 o = m.lst[k];
  if (m.rect) return t[o.x] * t[2 * m.nx + o.y] * t[2 * m.nx + 2 * m.ny + o.z];
  const SpheLayout L = sphe_layout(m.nmpol);
  const int l = o.x, mm = o.y;
  if (mm == 0) return t[L.ar() + l] * t[L.ap() + l * L.w];
  if (mm > 0) return t[L.ar() + l] * t[L.ac() + mm] * t[L.ap() + l * L.w + mm];
  return t[L.ar() + l] * t[L.as() - mm] * t[L.ap() + l * L.w - mm];
}

// Row of particle i in tab: the trial's row (index cap) stands in for
// particle j in INTERACT mode.
template <bool F32>
__global__ void __launch_bounds__(kMmThreads) k_mmij_tab(KP p, int mode) {
  const MmijDev &m = p.mm;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntot = p.st->ntot, i0 = p.nsites + p.nfix;
  double r[3], ist = 0.0;
  int row;
  if (mode == 1 && i == ntot) {  // INTERACT: the trial position
    const Trial tr = *p.trial;
    r[0] = tr.x;
    r[1] = tr.y;
    r[2] = tr.z;
    row = p.cap;
  } else {
    if (i >= ntot || i < i0) return;
    mm_pos<F32>(p, i, r);
    row = i;
  }
  double *t = m.tab + (size_t)row * m.tabw;
  const bool in = mm_tables(p, r, mode == 1 ? 1.0 : 10.0, t, ist);
  m.in[row] = in ? 1 : 0;
  m.ist[row] = ist;
}

// Chunk c of the ions: thread k sums q_i b_k(r_i) over the chunk.
__global__ void __launch_bounds__(kMmThreads) k_mmij_coef(KP p, int mode) {
  const MmijDev &m = p.mm;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (k >= m.ntpol) return;
  const int ntot = p.st->ntot, i0 = p.nsites + p.nfix;
  int j = -1;  // INTERACT: 0-based particle whose row is the trial's
  bool insert = false;
  int jtype = 0;
  if (mode == 1) {
    const Trial tr = *p.trial;
    j = tr.j - 1;
    insert = tr.insert;
    jtype = tr.itype;
  }
  const int iend = insert ? ntot + 1 : ntot;
  const int a = i0 + c * kMmChunk, b = min(iend, a + kMmChunk);
  double v = 0.0;
  for (int i = a; i < b; ++i) {
    const bool isj = mode == 1 && i == j;
    const int row = isj ? p.cap : i;
    if (!m.in[row]) continue;
    const double q = isj ? p.cg[jtype] : p.cg[abs(p.typei[i])];
    v += q * m.bnorm[k] * mm_value(m, k, m.tab + (size_t)row * m.tabw);
  }
  m.coefp[(size_t)c * m.ntpol + k] = v;
}

__global__ void __launch_bounds__(kMmThreads) k_mmij_sum(KP p, int mode, int nchunk) {
  const MmijDev &m = p.mm;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m.ntpol) {
    double v = 0.0;
    for (int c = 0; c < nchunk; ++c) v += m.coefp[(size_t)c * m.ntpol + k];
    m.coef[k] = v;
    if (mode == 1) {  // coef2 = coef - q_j b_k(r_j), j a mobile ion in the region
      const Trial tr = *p.trial;
      const int j = tr.j - 1, i0 = p.nsites + p.nfix;
      const bool jin = j >= i0 && m.in[p.cap];
      m.coef2[k] = jin ? v - p.cg[tr.itype] * m.bnorm[k] *
                                 mm_value(m, k, m.tab + (size_t)p.cap * m.tabw)
                       : v;
    }
  }
  if (mode == 0 && !m.rect && blockIdx.x == 0 && threadIdx.x == 0) {
    // sphe_rf1.f90's forces use the ist of the last ion in the sphere
    const int ntot = p.st->ntot;
    double ist = 0.0;
    for (int i = ntot - 1; i >= p.nsites + p.nfix; --i)
      if (m.in[i]) {
        ist = m.ist[i];
        break;
      }
    m.ist[p.cap + 1] = ist;
  }
}

// mode 0: mq_k = sum_l M_kl coef_l (x rfscal); mode 1: row k of
// E(coef) - E(coef2): (c_k^2 - c2_k^2) M_kk / 2 + sum_{l>k} (c_k c_l - c2_k c2_l) M_kl
__global__ void __launch_bounds__(kMmThreads) k_mmij_rows(KP p, int mode) {
  const MmijDev &m = p.mm;
  const int k = blockIdx.x * (kMmThreads / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= m.ntpol) return;
  const int n = m.ntpol;
  const double *row = m.m + (size_t)k * n;
  double v = 0.0;
  if (mode == 0) {
    for (int l = lane; l < n; l += 32) v += m.rect ? row[l] * m.coef[l] * m.rfscal : row[l] * m.coef[l];
  } else {
    const double ck = m.coef[k], c2k = m.coef2[k];
    for (int l = k + 1 + lane; l < n; l += 32) v += (ck * m.coef[l] - c2k * m.coef2[l]) * row[l];
    if (lane == 0) v += 0.5 * (ck * ck - c2k * c2k) * row[k];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) (mode == 0 ? m.mq : m.rowe)[k] = v;
}

// mode 0: egsbpb into energy slot `slot`; mode 1: INTERACT's term added to *dener
__global__ void __launch_bounds__(256) k_mmij_final(KP p, int mode, int slot, double *dener) {
  const MmijDev &m = p.mm;
  __shared__ double red[8];
  __shared__ double tot[1];
  double v[1] = {0.0};
  for (int k = threadIdx.x; k < m.ntpol; k += blockDim.x)
    v[0] += mode == 0 ? 0.5 * m.coef[k] * m.mq[k] : m.rowe[k];
  block_sum<1>(v, red, tot);
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    double *dst = p.epart + (size_t)slot * kNTerms;
    for (int k = 0; k < kNTerms; ++k) dst[k] = 0.0;
    dst[11] = tot[0] * p.celec;
  } else {
    *dener += m.rect ? tot[0] * p.celec * m.rfscal : tot[0] * p.celec;
  }
}

template <bool F32>
__global__ void __launch_bounds__(kMmThreads) k_mmij_force(KP p) {
  const MmijDev &m = p.mm;
  const int i = p.nsites + p.nfix + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.st->ntot || !m.in[i]) return;
  const double *t = m.tab + (size_t)i * m.tabw;
  double f[3] = {0.0, 0.0, 0.0};
  if (m.rect) {  // rect_rf1.f90:119-135
    const double *lx = t, *dlx = t + m.nx, *ly = t + 2 * m.nx, *dly = ly + m.ny;
    const double *lz = t + 2 * m.nx + 2 * m.ny, *dlz = lz + m.nz;
    for (int k = 0; k < m.ntpol; ++k) {
      const int3 o = m.lst[k];
      const double nrm = m.bnorm[k], mq = m.mq[k];
      const double xl = lx[o.x], yl = ly[o.y], zl = lz[o.z];
      f[0] -= nrm * dlx[o.x] * yl * zl * mq;
      f[1] -= nrm * xl * dly[o.y] * zl * mq;
      f[2] -= nrm * xl * yl * dlz[o.z] * mq;
    }
  } else {  // sphe_rf1.f90:120-160
    const SpheLayout L = sphe_layout(m.nmpol);
    const double *ar = t + L.ar(), *ac = t + L.ac(), *as = t + L.as();
    const double *ap = t + L.ap(), *adp = t + L.adp(), *ang = t + L.ang();
    const double st = ang[0], ct = ang[1], cp = ang[2], sp = ang[3];
    const double ist = m.ist[p.cap + 1];
    const int W = L.w;
    for (int k = 0; k < m.ntpol; ++k) {
      const int l = m.lst[k].x;
      int mm = m.lst[k].y;
      double dr = 0.0, ddt = 0.0, dp = 0.0;
      if (mm == 0) {
        if (l != 0) {
          const double rpl = ar[l - 1];
          dr = l * rpl * ap[l * W];
          ddt = -rpl * adp[l * W] * st;
        }
      } else if (mm > 0) {
        const double rpl = ar[l - 1], cmp = ac[mm], apl = ap[l * W + mm];
        dr = l * rpl * cmp * apl;
        ddt = -rpl * cmp * adp[l * W + mm] * st;
        dp = st == 0.0 ? 0.0 : -rpl * mm * as[mm] * apl * ist;
      } else {
        mm = -mm;
        const double rpl = ar[l - 1], smp = as[mm], apl = ap[l * W + mm];
        dr = l * rpl * smp * apl;
        ddt = -rpl * smp * adp[l * W + mm] * st;
        dp = st == 0.0 ? 0.0 : rpl * mm * ac[mm] * apl * ist;
      }
      const double nrm = m.bnorm[k], mq = m.mq[k];
      f[0] -= nrm * (dr * st * cp + ddt * ct * cp - dp * sp) * mq;
      f[1] -= nrm * (dr * st * sp + ddt * ct * sp + dp * cp) * mq;
      f[2] -= nrm * (dr * ct - ddt * st) * mq;
    }
  }
  const double ccc = p.cg[abs(p.typei[i])] * p.celec;
  const int cap = p.cap;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (F32)
      p.ffield_f[c * cap + i] += (float)(f[c] * ccc);
    else
      p.ffield[c * cap + i] += f[c] * ccc;
  }
}

int mmij_chunks(const KP &p, int ntot_ub) {
  return std::max(1, (std::max(0, ntot_ub + 1 - p.nsites - p.nfix) + kMmChunk - 1) / kMmChunk);
}

int launch_mmij(const KP &p, bool fp32, int ntot_ub, int qforces, int slot,
                cudaStream_t stream) {
  const MmijDev &m = p.mm;
  const int nion = std::max(0, ntot_ub - p.nsites - p.nfix);
  const int nt = m.ntpol, nch = mmij_chunks(p, ntot_ub);
  const int tb = (ntot_ub + kMmThreads - 1) / kMmThreads;
  if (tb > 0)
    (fp32 ? k_mmij_tab<true> : k_mmij_tab<false>)<<<tb, kMmThreads, 0, stream>>>(p, 0);
  k_mmij_coef<<<dim3((nt + kMmThreads - 1) / kMmThreads, nch), kMmThreads, 0, stream>>>(p, 0);
  k_mmij_sum<<<(nt + kMmThreads - 1) / kMmThreads, kMmThreads, 0, stream>>>(p, 0, nch);
  k_mmij_rows<<<(nt + kMmThreads / 32 - 1) / (kMmThreads / 32), kMmThreads, 0, stream>>>(p, 0);
  k_mmij_final<<<1, 256, 0, stream>>>(p, 0, slot, nullptr);
  int nk = 5;
  if (qforces && nion > 0) {
    (fp32 ? k_mmij_force<true> : k_mmij_force<false>)<<<(nion + kMmThreads - 1) / kMmThreads,
                                                        kMmThreads, 0, stream>>>(p);
    ++nk;
  }
  return nk;
}

void launch_mmij_interact(const KP &p, int ntot_ub, double *dener, cudaStream_t stream) {
  const MmijDev &m = p.mm;
  const int nt = m.ntpol, nch = mmij_chunks(p, ntot_ub);
  // positions are FP64 in INTERACT (the context keeps them current)
  k_mmij_tab<false><<<(ntot_ub + 1 + kMmThreads - 1) / kMmThreads, kMmThreads, 0, stream>>>(p, 1);
  k_mmij_coef<<<dim3((nt + kMmThreads - 1) / kMmThreads, nch), kMmThreads, 0, stream>>>(p, 1);
  k_mmij_sum<<<(nt + kMmThreads - 1) / kMmThreads, kMmThreads, 0, stream>>>(p, 1, nch);
  k_mmij_rows<<<(nt + kMmThreads / 32 - 1) / (kMmThreads / 32), kMmThreads, 0, stream>>>(p, 1);
  k_mmij_final<<<1, 256, 0, stream>>>(p, 1, 0, dener);
}

int mmij_table_width(int rect, int nx, int ny, int nz, int nmpol) {
  return rect ? 2 * (nx + ny + nz) : sphe_layout(nmpol).width();
}

}  // namespace bgpu
