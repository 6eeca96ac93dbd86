// Device bodies of the double-float HBS apply, shared by the per-level
// kernels (hbs_apply_df.cu) and the grouped kernels over many operators
// (group.cu).  Every float64 factor is a pair of float32 (hi, lo), x = hi + lo
// to 48 bits, and each multiply-accumulate is an error-free product (one
// fmaf) plus cross terms, added to the running (hi, lo) by TwoSum.
#pragma once

#include <cstdint>

namespace slu {
namespace dfk {

struct DF {
  float h, l;
};

__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float xh,
                                       float xl) {
  const float ph = __fmul_rn(ah, xh);
  float pl = __fmaf_rn(ah, xh, -ph);                  // exact product error
  pl = __fmaf_rn(ah, xl, __fmaf_rn(al, xh, pl));      // cross terms (al*xl dropped)
  const float s = __fadd_rn(sh, ph);                  // TwoSum(sh, ph)
  const float bb = __fsub_rn(s, sh);
  float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
  e = __fadd_rn(e, __fadd_rn(sl, pl));
  sh = __fadd_rn(s, e);                               // renormalise
  sl = __fsub_rn(e, __fsub_rn(sh, s));
}

__device__ __forceinline__ DF split_d(double x) {
  DF r;
  r.h = __double2float_rn(x);
  r.l = __double2float_rn(x - (double)r.h);
  return r;
}

constexpr int kBatch = 8;   // global loads in flight per thread in the copies

// Row/column of e = threadIdx.x + u * blockDim.x in a row-major array of
// `cols` columns, advanced without a division per element.
struct FlatIdx {
  int i, j, qs, rs, cols;
  __device__ FlatIdx(int cols_) : cols(cols_) {
    qs = blockDim.x / cols;
    rs = blockDim.x - qs * cols;
    i = threadIdx.x / cols;
    j = threadIdx.x - i * cols;
  }
  __device__ void next() {
    i += qs;
    j += rs;
    if (j >= cols) {
      j -= cols;
      ++i;
    }
  }
};

// Stage a rows x cols (hi, lo) block into shared memory with pitch ld.
__device__ inline void stage2(float* Sh, float* Sl, int ld, const float* __restrict__ Ah,
                              const float* __restrict__ Al, int rows, int cols) {
  const int total = rows * cols, step = blockDim.x;
  if (total == 0) return;
  FlatIdx ix(cols);
  for (int e0 = threadIdx.x; e0 < total; e0 += kBatch * step) {
    float h[kBatch], l[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int e = e0 + u * step;
      if (e < total) {
        h[u] = __ldg(Ah + e);
        l[u] = __ldg(Al + e);
      }
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (e0 + u * step < total) {
        Sh[ix.i * ld + ix.j] = h[u];
        Sl[ix.i * ld + ix.j] = l[u];
      }
      ix.next();
    }
  }
}

// (xh, xl)[i * ldx + cc] for i < rows, cc < nc: from the float64 X (rows
// perm[row0 + i], or row0 + i without perm), split into (hi, lo), or from the
// (hi, lo) pairs `in` (rows row0 + i, leading dimension c) when X is null.
__device__ inline void gather2(float* xh, float* xl, int ldx, const double* X, long long ldX,
                               const int64_t* __restrict__ perm, const DF* in, int c,
                               long long row0, int rows, int c0, int nc) {
  const int total = rows * nc, step = blockDim.x;
  if (total == 0) return;
  FlatIdx ix(nc);
  for (int e0 = threadIdx.x; e0 < total; e0 += kBatch * step) {
    FlatIdx at = ix;
    long long r[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const long long row = row0 + at.i;
      r[u] = (e0 + u * step < total && X && perm) ? __ldg(perm + row) : row;
      at.next();
    }
    DF v[kBatch];
    at = ix;
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (e0 + u * step < total)
        v[u] = X ? split_d(X[r[u] * ldX + c0 + at.j]) : in[r[u] * c + c0 + at.j];
      at.next();
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (e0 + u * step < total) {
        xh[ix.i * ldx + ix.j] = v[u].h;
        xl[ix.i * ldx + ix.j] = v[u].l;
      }
      ix.next();
    }
  }
}

// upward: out_b (k x c) = F_b^T in_b; leaf input from X (float64, perm gather)
__device__ __forceinline__ void df_up_body(float* smf, int b, int c0, int nc, int n, int k,
                                           const float* __restrict__ Fh,
                                           const float* __restrict__ Fl,
                                           const double* __restrict__ X, int ldx,
                                           const int64_t* __restrict__ perm,
                                           const DF* __restrict__ in, DF* __restrict__ out, int c,
                                           int cpb) {
  float* Sh = smf;                        // n x (k+1)
  float* Sl = Sh + n * (k + 1);
  float* xh = Sl + n * (k + 1);           // n x cpb
  float* xl = xh + n * cpb;
  gather2(xh, xl, cpb, X, ldx, perm, in, c, (long long)b * n, n, c0, nc);
  stage2(Sh, Sl, k + 1, Fh + (size_t)b * n * k, Fl + (size_t)b * n * k, n, k);
  __syncthreads();
  for (int e = threadIdx.x; e < k * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    float sh = 0.f, sl = 0.f;
    for (int j = 0; j < n; ++j)
      df_mac(sh, sl, Sh[j * (k + 1) + i], Sl[j * (k + 1) + i], xh[j * cpb + cc], xl[j * cpb + cc]);
    DF r;
    r.h = sh;
    r.l = sl;
    out[((size_t)b * k + i) * c + c0 + cc] = r;
  }
}

// downward / root: out_b = G_b uin_b + D_b vv_b; leaf: vv from X (perm gather),
// output float64 scattered through perm into Y.
__device__ __forceinline__ void df_down_body(float* smf, int b, int c0, int nc, int n, int k,
                                             const float* __restrict__ Gh,
                                             const float* __restrict__ Gl,
                                             const float* __restrict__ Dh,
                                             const float* __restrict__ Dl,
                                             const DF* __restrict__ uin,
                                             const DF* __restrict__ vv,
                                             const double* __restrict__ X, int ldx,
                                             const int64_t* __restrict__ perm,
                                             DF* __restrict__ out, double* __restrict__ Y, int ldy,
                                             int c, int cpb) {
  float* Sh = smf;                        // n x (n+1)
  float* Sl = Sh + n * (n + 1);
  float* xh = Sl + n * (n + 1);           // n x cpb
  float* xl = xh + n * cpb;
  float* uh = xl + n * cpb;               // k x cpb
  float* ul = uh + k * cpb;
  float* ah = ul + k * cpb;               // n x cpb accumulators
  float* al = ah + n * cpb;
  gather2(xh, xl, cpb, X, ldx, perm, vv, c, (long long)b * n, n, c0, nc);
  if (Gh) gather2(uh, ul, cpb, nullptr, 0, nullptr, uin, c, (long long)b * k, k, c0, nc);
  stage2(Sh, Sl, n + 1, Dh + (size_t)b * n * n, Dl + (size_t)b * n * n, n, n);
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    float sh = 0.f, sl = 0.f;
    const float* rh = Sh + i * (n + 1);
    const float* rl = Sl + i * (n + 1);
    for (int j = 0; j < n; ++j) df_mac(sh, sl, rh[j], rl[j], xh[j * cpb + cc], xl[j * cpb + cc]);
    ah[i * cpb + cc] = sh;
    al[i * cpb + cc] = sl;
  }
  if (Gh) {
    __syncthreads();
    stage2(Sh, Sl, k + 1, Gh + (size_t)b * n * k, Gl + (size_t)b * n * k, n, k);
    __syncthreads();
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
      int i = e / nc, cc = e - i * nc;
      float sh = ah[i * cpb + cc], sl = al[i * cpb + cc];
      const float* rh = Sh + i * (k + 1);
      const float* rl = Sl + i * (k + 1);
      for (int j = 0; j < k; ++j) df_mac(sh, sl, rh[j], rl[j], uh[j * cpb + cc], ul[j * cpb + cc]);
      ah[i * cpb + cc] = sh;
      al[i * cpb + cc] = sl;
    }
  }
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    long long row = (long long)b * n + i;
    if (Y) {
      Y[(perm ? perm[row] : row) * ldy + c0 + cc] =
          (double)ah[i * cpb + cc] + (double)al[i * cpb + cc];
    } else {
      DF r;
      r.h = ah[i * cpb + cc];
      r.l = al[i * cpb + cc];
      out[row * c + c0 + cc] = r;
    }
  }
}

}  // namespace dfk
}  // namespace slu
