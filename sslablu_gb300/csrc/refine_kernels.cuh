// Column norms and elementwise steps of the mixed-precision refinement,
// shared by the per-operator (refine.cu) and grouped (group.cu) loops.
#pragma once

#include "dfloat.cuh"

namespace slu {
namespace {

__global__ void colnorm2_k(int rows, int cols, const double* __restrict__ A, int lda,
                           double* __restrict__ out) {
  const int c = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    double v = A[(long long)i * lda + c];
    s += v * v;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    out[c] = t;
  }
}

// f = (float) src (dense, ld cols)
__global__ void to_f32_k(long long n, const double* __restrict__ src, float* __restrict__ f) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    f[e] = (float)src[e];
}

// x = f (init) or x += f
__global__ void accum_k(long long n, const float* __restrict__ f, double* __restrict__ x, int init) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    x[e] = init ? (double)f[e] : x[e] + (double)f[e];
}

// d = (double-float) src
__global__ void to_dfs_k(long long n, const double* __restrict__ src, dfloat* __restrict__ d) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    d[e] = to_dfloat(src[e]);
}

// x = d (init) or x += d
__global__ void accum_dfs_k(long long n, const dfloat* __restrict__ d, double* __restrict__ x,
                            int init) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const double v = to_double(d[e]);
    x[e] = init ? v : x[e] + v;
  }
}

// r = b - y (y double-float)
__global__ void resid_dfs_k(long long n, const double* __restrict__ b, const dfloat* __restrict__ y,
                            double* __restrict__ r) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const dfloat v = y[e];
    r[e] = (b[e] - (double)v.h) - (double)v.l;
  }
}

// x += d
__global__ void add_k(long long n, const double* __restrict__ d, double* __restrict__ x) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    x[e] += d[e];
}

// out[j] += sum_i A_ij^2 for a rows x cols row-major block: one thread per
// column (consecutive threads read consecutive columns: coalesced), rows
// split over blockIdx.y; out zeroed by the caller.
__global__ void colsumsq_k(int rows, int cols, const double* __restrict__ A, int lda,
                           double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const int per = (rows + gridDim.y - 1) / gridDim.y;
  const int i0 = blockIdx.y * per, i1 = min(rows, i0 + per);
  double s = 0.0;
  for (int i = i0; i < i1; ++i) {
    const double v = A[(long long)i * lda + j];
    s = fma(v, v, s);
  }
  if (i1 > i0) atomicAdd(out + j, s);
}

// r = b - r
__global__ void resid_k(long long n, const double* __restrict__ b, double* __restrict__ r) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    r[e] = b[e] - r[e];
}

inline int gsz(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

}  // namespace
}  // namespace slu
