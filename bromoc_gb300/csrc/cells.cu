// Cell list of the periodic extension mode, FP32 path, and the pair kernel
// that walks it.  The reference evaluates every ion pair
// (energy.mono.f90:117-194); the extension mode adds a minimum-image box and
// a plain cutoff rc, and with a cutoff only the pairs within rc count.  The
// box is cut into cells of edge at least rc (1 + 1e-4): a pair within rc then
// always lies in the same or a neighbouring cell, even when rounding puts an
// ion near a cell face on the other side of it.
//
// Built on the device every energy evaluation (the ions move every step):
//   count  : each ion's cell from its float-float position, counts per cell;
//   scan   : exclusive prefix sum of the counts (one block);
//   fill   : ions into their cell's stretch (atomic cursor per cell);
//   sort   : each cell's stretch in ascending ion order (one thread per
//            cell), so a run always sums a particle's pairs in one order.
// Pair kernel: kCellLanes lanes per ion, in cell order (the lanes of a
// warp mostly share their 27 neighbour cells, so the source records they
// read coincide); lane u of an ion takes every kCellLanes-th candidate of
// each neighbour cell, and the lanes' sums meet in a fixed shuffle tree.
// Each pair is evaluated by both of its ions, weight 1/2 per mobile source,
// the conventions of the chunked kernel k_pairs32 (FP32 partials fii_f,
// chunk 0; block partial energies).  Used when every axis holds at least four
// cells; smaller boxes keep the all-pairs Newton-3 tile.
#include <algorithm>

#include "launch.h"
#include "pairs_n3.cuh"

namespace bgpu {

constexpr int kCellThreads = 256;
constexpr int kCellLanes = 4;  // lanes per ion in the pair kernel

__device__ __forceinline__ int cell_of(const KP &p, const float4 &h, const float4 &l) {
  const float hh[3] = {h.x, h.y, h.z}, ll[3] = {l.x, l.y, l.z};
  int c[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float u = ((hh[a] - p.f.box.bh[2 * a]) + (ll[a] - p.f.box.bl[2 * a])) * p.cinv[a];
    c[a] = min(max((int)floorf(u), 0), p.nc[a] - 1);
  }
  return (c[0] * p.nc[1] + c[1]) * p.nc[2] + c[2];
}

__global__ void __launch_bounds__(kCellThreads) k_cell_count(KP p) {
  const int i = p.nsites + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.st->ntot) return;
  const int c = cell_of(p, p.pk1[i], p.pk2[i]);
  p.ion_cell[i] = c;
  atomicAdd(p.cell_n + c, 1);
}

// Exclusive prefix sum of the counts into cell_start[0..ncells]; the counts
// are cleared for their use as cursors.  One block of 1024 threads, each
// over a contiguous run of cells.
__global__ void __launch_bounds__(1024) k_cell_scan(KP p) {
  __shared__ int part[1024];
  const int n = p.ncells, per = (n + 1023) / 1024;
  const int b0 = min(n, (int)threadIdx.x * per), b1 = min(n, b0 + per);
  int s = 0;
  for (int c = b0; c < b1; ++c) s += p.cell_n[c];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive scan of the run totals
    const int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int c = b0; c < b1; ++c) {
    const int k = p.cell_n[c];
    p.cell_start[c] = run;
    run += k;
    p.cell_n[c] = 0;
  }
  if (threadIdx.x == 1023) p.cell_start[n] = part[1023];
}

__global__ void __launch_bounds__(kCellThreads) k_cell_fill(KP p) {
  const int i = p.nsites + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.st->ntot) return;
  const int c = p.ion_cell[i];
  p.cell_ion[p.cell_start[c] + atomicAdd(p.cell_n + c, 1)] = i;
}

__global__ void __launch_bounds__(kCellThreads) k_cell_sort(KP p) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= p.ncells) return;
  int *v = p.cell_ion + p.cell_start[c];
  const int n = p.cell_start[c + 1] - p.cell_start[c];
  for (int a = 1; a < n; ++a) {  // insertion sort: a cell holds tens of ions
    const int x = v[a];
    int b = a - 1;
    while (b >= 0 && v[b] > x) {
      v[b + 1] = v[b];
      --b;
    }
    v[b + 1] = x;
  }
}

template <bool EFP>
__global__ void __launch_bounds__(kCellThreads) k_pairs_cell(KP p, int qforces, int slot0) {
  __shared__ float4 tab[EFP ? 1 : kIpqMax];
  __shared__ float red[(kCellThreads / 32) * 4];
  __shared__ float tot[4];
  const int nt = p.nion_t;
  if (!EFP)
    for (int k = threadIdx.x; k < nt * ipq_stride(nt); k += blockDim.x) tab[k] = __ldg(p.ipq + k);
  __syncthreads();
  const int ntot = p.st->ntot, m0 = p.nsites + p.nfix;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = t / kCellLanes, u = t % kCellLanes;
  const int i = k < ntot - p.nsites ? p.cell_ion[k] : -1;
  float fx = 0.f, fy = 0.f, fz = 0.f;
  float e[4] = {0.f, 0.f, 0.f, 0.f};  // ecoul, elj (6 x elj with the dense table), esrpmf, eefpot
  if (i >= m0) {  // mobile target
    const float4 th = p.pk1[i], tl = p.pk2[i];
    const int tcode = __float_as_int(th.w);
    const int row =
        EFP ? (tcode & 0xffff) * p.nttyp : ((tcode & 0xffff) - p.ndna) * ipq_stride(nt);
    const int c = p.ion_cell[i];
    const int n1 = p.nc[1], n2 = p.nc[2];
    const int cz = c % n2, cy = (c / n2) % n1, cx = c / (n1 * n2);
    for (int ox = -1; ox <= 1; ++ox) {
      int ax = cx + ox;
      ax += ax < 0 ? p.nc[0] : 0;
      ax -= ax >= p.nc[0] ? p.nc[0] : 0;
      for (int oy = -1; oy <= 1; ++oy) {
        int ay = cy + oy;
        ay += ay < 0 ? n1 : 0;
        ay -= ay >= n1 ? n1 : 0;
        for (int oz = -1; oz <= 1; ++oz) {
          int az = cz + oz;
          az += az < 0 ? n2 : 0;
          az -= az >= n2 ? n2 : 0;
          const int cc = (ax * n1 + ay) * n2 + az;
          const int s1 = p.cell_start[cc + 1];
          for (int s = p.cell_start[cc] + u; s < s1; s += kCellLanes) {
            const int j = p.cell_ion[s];
            if (j == i) continue;
            const float4 h = p.pk1[j], l = p.pk2[j];
            float dx = (th.x - h.x) + (tl.x - l.x);
            float dy = (th.y - h.y) + (tl.y - l.y);
            float dz = (th.z - h.z) + (tl.z - l.z);
            min_image_f(p, dx, dy, dz);
            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (r2 >= p.f.rc2) continue;
            const int code = __float_as_int(h.w);
            const float w = (code >> 16) ? 0.5f : 1.0f;
            float de;
            if (EFP) {
              de = law32k(p, __ldg(p.pidx + row + (code & 0xffff)), r2, w, e,
                          [&] { return pair_r2_64<true>(p, th, tl, h, l); });
            } else {
              const float4 q = tab[row + (code & 0xffff) - p.ndna];
              const float ir = rsqrt_nz(r2), ir2 = ir * ir;
              const float cofo = q.x * ir;
              e[0] = fmaf(w, cofo, e[0]);
              float d6 = q.z * ir2;
              d6 = d6 * d6 * d6;
              const float d12 = d6 * d6;
              e[1] = fmaf(w, q.y * (d12 - d6), e[1]);
              de = ir2 * fmaf(q.y, fmaf(2.0f, d12, -d6), cofo);
              if (r2 <= q.w)
                de += srpmf32(p, srp_index(p, tcode, code), r2, ir, w, e,
                              srp_branch(p, r2, [&] { return pair_r2_64<true>(p, th, tl, h, l); }));
            }
            fx = fmaf(de, dx, fx);
            fy = fmaf(de, dy, fy);
            fz = fmaf(de, dz, fz);
          }
        }
      }
    }
  }
#pragma unroll
  for (int o = 1; o < kCellLanes; o <<= 1) {  // the ion's lanes, fixed order
    fx += __shfl_xor_sync(0xffffffffu, fx, o);
    fy += __shfl_xor_sync(0xffffffffu, fy, o);
    fz += __shfl_xor_sync(0xffffffffu, fz, o);
  }
  if (i >= 0 && u == 0) {
    float *f = p.fii_f;  // chunk 0
    f[i] = qforces ? fx : 0.f;
    f[p.cap + i] = qforces ? fy : 0.f;
    f[2 * p.cap + i] = qforces ? fz : 0.f;
  }
  block_sum_f<4>(e, red, tot);
  if (threadIdx.x == 0) {
    double *dst = p.epart + (size_t)(slot0 + blockIdx.x) * kNTerms;
    for (int m = 0; m < kNTerms; ++m) dst[m] = 0.0;
    dst[1] = tot[0];
    dst[2] = EFP ? (double)tot[1] : (double)tot[1] / 6.0;
    dst[3] = tot[2];
    dst[4] = tot[3];
  }
}

int cell_pair_blocks(const KP &p, int ntot_ub) {
  return (std::max(0, ntot_ub - p.nsites) * kCellLanes + kCellThreads - 1) / kCellThreads;
}

int launch_cells(const KP &p, int ntot_ub, int qforces, int slot, cudaStream_t stream) {
  const int nion = std::max(0, ntot_ub - p.nsites);
  if (nion == 0 || p.ncells <= 0) return 0;
  const int nb = (nion + kCellThreads - 1) / kCellThreads;
  cudaMemsetAsync(p.cell_n, 0, (size_t)(p.ncells + 1) * sizeof(int), stream);
  k_cell_count<<<nb, kCellThreads, 0, stream>>>(p);
  k_cell_scan<<<1, 1024, 0, stream>>>(p);
  k_cell_fill<<<nb, kCellThreads, 0, stream>>>(p);
  k_cell_sort<<<(p.ncells + kCellThreads - 1) / kCellThreads, kCellThreads, 0, stream>>>(p);
  const int npb = cell_pair_blocks(p, ntot_ub);
  if (p.ipq_ok)
    k_pairs_cell<false><<<npb, kCellThreads, 0, stream>>>(p, qforces, slot);
  else
    k_pairs_cell<true><<<npb, kCellThreads, 0, stream>>>(p, qforces, slot);
  return 5;
}

}  // namespace bgpu
