// Float-float arithmetic of the FP32 path.  GB300 runs FP64 at a small
// fraction of its FP32 rate, so in FP32 mode a particle position is carried
// as an unevaluated sum hi + lo of two floats (about 48 significant bits,
// ~1e-12 A at 100 A) and every per-step kernel stays on the FP32 pipe.  The
// FP64 coordinate arrays are refreshed from these pairs only where FP64 code
// (GCMC, the host API) reads them.
//
// two_sum / fast_two_sum are the error-free transformations of Knuth and
// Dekker; they rely on IEEE round-to-nearest float arithmetic without
// reassociation (the build uses no fast-math flags).
#pragma once
#include "kparams.cuh"

namespace bgpu {

// s + e == a + b exactly, s = fl(a + b)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// as two_sum, for |a| >= |b|
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// (h, l) += d, renormalised so that |l| <= ulp(h) / 2
__device__ __forceinline__ void ff_add(float &h, float &l, float d) {
  float s, e;
  two_sum(h, d, s, e);
  e = __fadd_rn(e, l);
  fast_two_sum(s, e, h, l);
}

// (ah + al) - (bh + bl), rounded to float; exact high part when ah ~ bh
__device__ __forceinline__ float ff_diff(float ah, float al, float bh, float bl) {
  return __fadd_rn(__fsub_rn(ah, bh), __fsub_rn(al, bl));
}

// compensated accumulation: (s, c) += v
__device__ __forceinline__ void acc2(float &s, float &c, float v) {
  float e;
  two_sum(s, v, s, e);
  c = __fadd_rn(c, e);
}

// (s1, c1) += (s2, c2)
__device__ __forceinline__ void acc2p(float &s1, float &c1, float s2, float c2) {
  float e;
  two_sum(s1, s2, s1, e);
  c1 = __fadd_rn(__fadd_rn(c1, c2), e);
}

// Grid cell of one coordinate in float-float: xi = pos + (tran - cen),
// ix = int(xi / dcel) (trunc) or nint(xi / dcel) (spline stencil), and the
// offset r = xi - ix dcel.  The first guess of ix comes from a rounded
// quotient; the exactly rounded remainder then corrects it by one cell, so
// ix agrees with the double-precision index except within ~1e-7 dcel of a
// cell face.  Returns u - ix = r / dcel.
__device__ __forceinline__ float ff_cell(const AxisF &A, float ph, float pl,
                                         bool nint, int &ix) {
  float s, e;
  two_sum(ph, A.oh, s, e);
  const float t = __fadd_rn(__fadd_rn(pl, A.ol), e);  // xi = s + t
  const float u0 = __fmul_rn(__fadd_rn(s, t), A.idc);
  ix = nint ? (int)copysignf(floorf(fabsf(u0) + 0.5f), u0) : (int)u0;
  const float fx = (float)ix;
  float r = fmaf(-fx, A.dh, s);
  r = __fadd_rn(fmaf(-fx, A.dl, r), t);
  if (nint) {  // nint(u), then the reference's clamps (vdwgd1spln.f90:98-107)
    const float half = 0.5f * A.dh;
    if (r < -half) {
      --ix;
      r = __fadd_rn(r, A.dh);
    } else if (r >= half) {
      ++ix;
      r = __fsub_rn(r, A.dh);
    }
    if (ix == 0) {
      ix = 1;
      r = __fsub_rn(r, A.dh);
    }
    if (ix == A.ncl - 1) {
      ix = A.ncl - 2;
      r = __fadd_rn(r, A.dh);
    }
  } else {  // int(u) for u >= 0, then the far-face clamp (staticf1.f90:70-75)
    if (u0 >= 0.0f) {
      if (r < 0.0f && ix > 0) {
        --ix;
        r = __fadd_rn(r, A.dh);
      } else if (r >= A.dh) {
        ++ix;
        r = __fsub_rn(r, A.dh);
      }
    }
    if (ix == A.ncl - 1) {
      ix = A.ncl - 2;
      r = __fadd_rn(r, A.dh);
    }
  }
  return __fmul_rn(r, A.idc);
}

// lb <= pos <= ub in float-float
__device__ __forceinline__ bool ff_inside(const AxisF &A, float ph, float pl) {
  return ff_diff(ph, pl, A.ubh, A.ubl) <= 0.0f && ff_diff(ph, pl, A.lbh, A.lbl) >= 0.0f;
}

// Fixed-tree block sum in float; totals land in the shared array out[N].
// smem: (blockDim.x/32) * N floats.
template <int N>
__device__ __forceinline__ void block_sum_f(const float v[N], float *smem, float *out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    float x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) smem[wid * N + k] = x;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    float s = 0.0f;
    for (int w = 0; w < nw; ++w) s += smem[w * N + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

__device__ __forceinline__ void clamp_f(float bdmax, float &d) {
  if (fabsf(d) > bdmax) d = copysignf(bdmax, d);
}

// (h, l) += (ah, al), renormalised
__device__ __forceinline__ void ff_add2(float &h, float &l, float ah, float al) {
  float s, e;
  two_sum(h, ah, s, e);
  e = __fadd_rn(e, __fadd_rn(l, al));
  fast_two_sum(s, e, h, l);
}

// fixcoor.f90:19-68 on float-float coordinates; in the extension mode
// (periodic box) one wrap into [lower bound, lower bound + L) per axis.
__device__ __forceinline__ void fixcoor_ff(const BoxF &c, float h[3], float l[3]) {
  if (c.periodic) {
    for (int k = 0; k < 3; ++k) {
      if (ff_diff(h[k], l[k], c.bh[2 * k], c.bl[2 * k]) < 0.0f)
        ff_add2(h[k], l[k], c.Lh[k], c.Ll[k]);
      else if (ff_diff(h[k], l[k], c.bh[2 * k + 1], c.bl[2 * k + 1]) >= 0.0f)
        ff_add2(h[k], l[k], -c.Lh[k], -c.Ll[k]);
    }
    return;
  }
  if (c.shape == 1) {  // sphere: reflect through the wall
    const float d0 = ff_diff(h[0], l[0], c.ch[0], c.cl[0]);
    const float d1 = ff_diff(h[1], l[1], c.ch[1], c.cl[1]);
    const float d2 = ff_diff(h[2], l[2], c.ch[2], c.cl[2]);
    const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
    if (r2 > c.rsphe2) {
      const float lzrad = 2.0f * c.rsphe * rsqrtf(r2) - 1.0f;
      const float d[3] = {d0, d1, d2};
      for (int k = 0; k < 3; ++k) {
        h[k] = c.ch[k];
        l[k] = c.cl[k];
        ff_add(h[k], l[k], lzrad * d[k]);
      }
    }
    return;
  }
  int k0 = 0;
  if (c.shape == 2) {  // elliptic cylinder
    const float ex = ff_diff(h[0], l[0], c.ch[0], c.cl[0]) * c.iecx;
    const float ey = ff_diff(h[1], l[1], c.ch[1], c.cl[1]) * c.iecy;
    const float r2 = fmaf(ex, ex, ey * ey);
    if (r2 > 1.0f) {
      const float r = 0.99999994f * rsqrtf(r2);
      for (int k = 0; k < 2; ++k) {
        const float d = ff_diff(h[k], l[k], c.ch[k], c.cl[k]);
        h[k] = c.ch[k];
        l[k] = c.cl[k];
        ff_add(h[k], l[k], r * d);
      }
    }
    k0 = 2;
  }
  for (int k = k0; k < 3; ++k) {  // box clamp (z only for the cylinder)
    if (ff_diff(h[k], l[k], c.bh[2 * k], c.bl[2 * k]) < 0.0f) {
      h[k] = c.bh[2 * k];
      l[k] = c.bl[2 * k];
    } else if (ff_diff(h[k], l[k], c.bh[2 * k + 1], c.bl[2 * k + 1]) > 0.0f) {
      h[k] = c.bh[2 * k + 1];
      l[k] = c.bl[2 * k + 1];
    }
  }
}

}  // namespace bgpu
