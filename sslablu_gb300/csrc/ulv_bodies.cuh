// Device bodies of the fused ULV solve (mode N), shared by the per-level
// kernels (ulv_solve.cu) and the grouped kernels over many operators
// (group.cu).  Arithmetic of ULVsparse.solve (matAssembly/HBS/
// ULVsparse.py:296-327):
//   forward, level t (leaf -> root-1):  z = Q_b^T x_b, the leading nu rows are
//     kept (ru), the trailing k rows form the parent's input;
//   root:  y = R^{-1} (Q^T x),  v = D y;
//   backward, level t (root-1 -> leaf):
//     y_u  = R11^{-1} (ru - Uu v - R12 y_next)
//     ynew = W [y_u; y_next],  vnew = U v + D ynew
// Each body is run by one CTA on block b and right-hand-side columns
// [c0, c0 + nc); shared memory is laid out per body (see the comments).
#pragma once

#include <cstdint>

namespace slu {
namespace ulvk {


// Global -> shared copies keep kBatch loads in flight per thread: issued as
// one group, then stored, so a copy of e elements costs about
// e / (kBatch * blockDim) memory round trips instead of e / blockDim.
constexpr int kBatch = 8;

// Row/column of the flat index e = threadIdx.x + u * blockDim.x, u = 0, 1,
// ..., in a row-major array of `cols` columns, advanced without a division
// per element (one division per thread at the start).
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

// S[i * ld + j] = A[i * cols + j], a rows x cols block.
template <typename T>
__device__ inline void stage(T* S, int ld, const T* __restrict__ A, int rows, int cols) {
  const int total = rows * cols, step = blockDim.x;
  if (total == 0) return;
  FlatIdx ix(cols);
  for (int e0 = threadIdx.x; e0 < total; e0 += kBatch * step) {
    T v[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int e = e0 + u * step;
      if (e < total) v[u] = __ldg(A + e);
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (e0 + u * step < total) S[ix.i * ld + ix.j] = v[u];
      ix.next();
    }
  }
}

// x[i * ldx + cc] = src[r_i * lds + c0 + cc] for i < rows, cc < nc, with
// r_i = perm[row0 + i] when perm is given, else row0 + i.
template <typename T>
__device__ inline void gather(T* x, int ldx, const T* src, long long lds,
                              const int64_t* __restrict__ perm, long long row0, int rows,
                              int c0, int nc) {
  const int total = rows * nc, step = blockDim.x;
  if (total == 0) return;
  FlatIdx ix(nc);
  for (int e0 = threadIdx.x; e0 < total; e0 += kBatch * step) {
    FlatIdx at = ix;
    long long r[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const long long row = row0 + at.i;
      r[u] = (e0 + u * step < total && perm) ? __ldg(perm + row) : row;
      at.next();
    }
    T v[kBatch];
    at = ix;
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      // L2-only loads: in a persistent kernel the same buffer is rewritten
      // by other SMs between steps, so no stale L1 line may be used
      if (e0 + u * step < total) v[u] = __ldcg(src + r[u] * lds + c0 + at.j);
      at.next();
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (e0 + u * step < total) x[ix.i * ldx + ix.j] = v[u];
      ix.next();
    }
  }
}

// B[perm[row0 + i] * ldb + c0 + cc] = y[i * ldy + cc] for i < rows, cc < nc,
// with the permutation loads batched.
template <typename T>
__device__ inline void scatter(T* B, long long ldb, const int64_t* __restrict__ perm,
                               long long row0, const T* y, int ldy, int rows, int c0, int nc) {
  const int total = rows * nc, step = blockDim.x;
  if (total == 0) return;
  FlatIdx ix(nc);
  for (int e0 = threadIdx.x; e0 < total; e0 += kBatch * step) {
    FlatIdx at = ix;
    long long r[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      r[u] = (e0 + u * step < total) ? __ldg(perm + row0 + at.i) : 0;
      at.next();
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (e0 + u * step < total) B[r[u] * ldb + c0 + ix.j] = y[ix.i * ldy + ix.j];
      ix.next();
    }
  }
}

// Asynchronous global -> shared copies (cp.async, Ampere and later): every
// element of every block matrix a CTA needs can be in flight at once, and one
// wait covers them all.  The wait is the hardware's completion of the
// thread's own copies.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  if (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// S[i * ld + j] <- A[i * cols + j] as asynchronous copies (complete after
// cp_async_wait_all and a barrier).
template <typename T>
__device__ inline void stage_async(T* S, int ld, const T* A, int rows, int cols) {
  const int total = rows * cols;
  if (total == 0) return;
  FlatIdx ix(cols);
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    cp_async_elem(S + ix.i * ld + ix.j, A + e);
    ix.next();
  }
}

// Dot products of the matrix-vector steps are split over ks consecutive lanes
// (each sums every ks-th term, then a butterfly of shuffles adds the ks
// partial sums): the dependent multiply-add chain is ks times shorter and
// more lanes work when there are few columns.  ks depends only on the
// length of the dot product, so the summation order -- and the result --
// does not depend on how the right-hand sides are chunked over CTAs.
__device__ __forceinline__ int dot_split(int len) { return len >= 32 ? 4 : (len >= 8 ? 2 : 1); }

// out[i][c] (+)= sign * sum_j S[i][j0 + j] * x[j][c]   i < rows, j < cols
template <typename T>
__device__ inline void mv(const T* S, int ld, int j0, int rows, int cols, const T* x, int ldx,
                          T* out, int ldo, int nc, T sign, bool accumulate) {
  const int ks = dot_split(cols), lks = ks == 4 ? 2 : (ks == 2 ? 1 : 0);
  const int work = rows * nc * ks, lane = threadIdx.x & 31;
  for (int base = threadIdx.x - lane; base < work; base += blockDim.x) {
    const int t = base + lane;
    const bool on = t < work;
    const int e = t >> lks, part = t & (ks - 1);
    const int i = on ? e / nc : 0, cc = on ? e - i * nc : 0;
    T acc = T(0);
    if (on) {
      const T* s = S + i * ld + j0;
#pragma unroll 4
      for (int j = part; j < cols; j += ks) acc = fma(s[j], x[j * ldx + cc], acc);
    }
    for (int o = ks >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (on && part == 0) {
      T* op = out + i * ldo + cc;
      *op = accumulate ? fma(sign, acc, *op) : sign * acc;
    }
  }
}

// out[i][c] = sum_j S[j][i] * x[j][c]   (transposed product)
template <typename T>
__device__ inline void mvt(const T* S, int ld, int rows_out, int cols_in, const T* x, int ldx,
                           T* out, int ldo, int nc) {
  const int ks = dot_split(cols_in), lks = ks == 4 ? 2 : (ks == 2 ? 1 : 0);
  const int work = rows_out * nc * ks, lane = threadIdx.x & 31;
  for (int base = threadIdx.x - lane; base < work; base += blockDim.x) {
    const int t = base + lane;
    const bool on = t < work;
    const int e = t >> lks, part = t & (ks - 1);
    const int i = on ? e / nc : 0, cc = on ? e - i * nc : 0;
    T acc = T(0);
    if (on) {
#pragma unroll 4
      for (int j = part; j < cols_in; j += ks) acc = fma(S[j * ld + i], x[j * ldx + cc], acc);
    }
    for (int o = ks >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (on && part == 0) out[i * ldo + cc] = acc;
  }
}

// x <- R^{-1} x for the leading m x m upper triangle of staged R (pitch ld).
// The diagonal of the staged copy is replaced by its reciprocals (all threads,
// once), then one warp per right-hand-side column runs the back substitution:
// lane (i mod 32) finishes x_i and broadcasts it, each lane updates the rows
// it owns (r = lane + 32 q).  Rows never change owner, so the sweep needs no
// block barrier.
template <typename T>
__device__ inline void trsv_upper(T* R, int ld, int m, T* x, int ldx, int nc) {
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) R[i * ld + i] = T(1) / R[i * ld + i];
  __syncthreads();
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int cc = threadIdx.x >> 5; cc < nc; cc += nw) {
    for (int i = m - 1; i >= 0; --i) {
      const int owner = i & 31;
      T xi = T(0);
      if (lane == owner) {
        xi = x[i * ldx + cc] * R[i * ld + i];
        x[i * ldx + cc] = xi;
      }
      xi = __shfl_sync(0xffffffffu, xi, owner);
      for (int r = lane; r < i; r += 32) x[r * ldx + cc] -= R[r * ld + i] * xi;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- forward
template <typename T>
__device__ __forceinline__ void ulv_fwd_body(unsigned char* sm_raw, int b, int c0, int nc, int n,
                                             int nu, int k, const T* __restrict__ Q,
                                             const T* __restrict__ src, int lds,
                                             const int64_t* __restrict__ perm, T* __restrict__ ru,
                                             T* __restrict__ dst, int c, int cpb) {
  T* S = reinterpret_cast<T*>(sm_raw);       // n x (n+1)
  T* x = S + n * (n + 1);                     // n x cpb
  T* z = x + n * cpb;                         // n x cpb
  stage_async(S, n + 1, Q + (size_t)b * n * n, n, n);
  gather(x, cpb, src, lds, perm, (long long)b * n, n, c0, nc);
  cp_async_wait_all();
  __syncthreads();
  mvt(S, n + 1, n, n, x, cpb, z, cpb, nc);
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    T v = z[i * cpb + cc];
    if (i < nu) ru[((size_t)b * nu + i) * c + c0 + cc] = v;
    else dst[((size_t)b * k + (i - nu)) * c + c0 + cc] = v;
  }
}

// ---------------------------------------------------------------- root
// y = R^{-1} Q^T x, v = D y.  When the tree has one level the root is also
// the leaf: input gathered through perm, solution scattered through perm.
// Shared memory: with PF, Q, R and D (n x (n+1) each) copied in one
// asynchronous batch; without PF one n x (n+1) region restaged per matrix.
// Then x, y (n x cpb each).
template <typename T, bool PF>
__device__ __forceinline__ void ulv_root_body(unsigned char* sm_raw, int c0, int nc, int n,
                                              const T* __restrict__ Q, const T* __restrict__ R,
                                              const T* __restrict__ D, const T* __restrict__ src,
                                              int lds, const int64_t* __restrict__ perm,
                                              T* __restrict__ Yout, T* __restrict__ Vout,
                                              T* __restrict__ B, int ldb, int c, int cpb) {
  T* SQ = reinterpret_cast<T*>(sm_raw);
  T* SR = PF ? SQ + n * (n + 1) : SQ;
  T* SD = PF ? SR + n * (n + 1) : SQ;
  T* x = (PF ? SD : SQ) + n * (n + 1);
  T* y = x + n * cpb;
  stage_async(SQ, n + 1, Q, n, n);
  if (PF) {
    stage_async(SR, n + 1, R, n, n);
    if (!perm) stage_async(SD, n + 1, D, n, n);
  }
  gather(x, cpb, src, lds, perm, 0, n, c0, nc);
  cp_async_wait_all();
  __syncthreads();
  mvt(SQ, n + 1, n, n, x, cpb, y, cpb, nc);
  if (!PF) {
    __syncthreads();
    stage(SR, n + 1, R, n, n);
  }
  trsv_upper(SR, n + 1, n, y, cpb, nc);   // begins and ends with a barrier
  if (perm) {  // single-level tree: y is the solution
    scatter(B, ldb, perm, 0, y, cpb, n, c0, nc);
    return;
  }
  if (!PF) {
    stage(SD, n + 1, D, n, n);
    __syncthreads();
  }
  mv(SD, n + 1, 0, n, n, y, cpb, x, cpb, nc, T(1), false);   // x <- D y
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    Yout[(size_t)i * c + c0 + cc] = y[i * cpb + cc];
    Vout[(size_t)i * c + c0 + cc] = x[i * cpb + cc];
  }
}

// ---------------------------------------------------------------- backward
// Shared memory (elements of T): with PF every block matrix has its own
// region -- Uu nu x (k+1), R nu x (n+1), W n x (n+1) and, above the leaves,
// U n x (k+1), D n x (n+1) -- all copied in one asynchronous batch; without
// PF one n x (n+1) region is restaged per matrix.  Then vb, yn (k x cpb),
// yu (nu x cpb), ynew and vt (n x cpb).
template <typename T, bool PF>
__device__ __forceinline__ void ulv_bwd_body(unsigned char* sm_raw, int b, int c0, int nc, int n,
                                             int nu, int k, const T* __restrict__ ru,
                                             const T* __restrict__ Uu, const T* __restrict__ R,
                                             const T* __restrict__ W, const T* __restrict__ U,
                                             const T* __restrict__ D, const T* __restrict__ Vin,
                                             const T* __restrict__ Yin, T* __restrict__ Yout,
                                             T* __restrict__ Vout, const int64_t* __restrict__ perm,
                                             T* __restrict__ B, int ldb, int c, int cpb) {
  const bool leaf = perm != nullptr;
  T* base = reinterpret_cast<T*>(sm_raw);
  T *SUu = base, *SR = base, *SW = base, *SU = base, *SD = base, *vec;
  if (PF) {
    SR = SUu + nu * (k + 1);
    SW = SR + nu * (n + 1);
    SU = SW + n * (n + 1);
    SD = SU + (leaf ? 0 : n * (k + 1));
    vec = SD + (leaf ? 0 : n * (n + 1));
    if (nu > 0) {
      stage_async(SUu, k + 1, Uu + (size_t)b * nu * k, nu, k);
      stage_async(SR, n + 1, R + (size_t)b * nu * n, nu, n);
    }
    stage_async(SW, n + 1, W + (size_t)b * n * n, n, n);
    if (!leaf) {
      stage_async(SU, k + 1, U + (size_t)b * n * k, n, k);
      stage_async(SD, n + 1, D + (size_t)b * n * n, n, n);
    }
  } else {
    vec = base + n * (n + 1);
  }
  T* vb = vec;                 // k  x cpb
  T* yn = vb + k * cpb;        // k  x cpb
  T* yu = yn + k * cpb;        // nu x cpb
  T* ynew = yu + nu * cpb;     // n  x cpb
  T* vt = ynew + n * cpb;      // n  x cpb
  gather(vb, cpb, Vin, c, nullptr, (long long)b * k, k, c0, nc);
  gather(yn, cpb, Yin, c, nullptr, (long long)b * k, k, c0, nc);
  gather(yu, cpb, ru, c, nullptr, (long long)b * nu, nu, c0, nc);
  if (PF) cp_async_wait_all();
  if (nu > 0) {
    // yu = ru - Uu v - R12 y_next ; then R11^{-1}
    if (!PF) stage(SUu, k + 1, Uu + (size_t)b * nu * k, nu, k);
    __syncthreads();
    mv(SUu, k + 1, 0, nu, k, vb, cpb, yu, cpb, nc, T(-1), true);
    __syncthreads();
    if (!PF) {
      stage(SR, n + 1, R + (size_t)b * nu * n, nu, n);
      __syncthreads();
    }
    mv(SR, n + 1, nu, nu, k, yn, cpb, yu, cpb, nc, T(-1), true);
    trsv_upper(SR, n + 1, nu, yu, cpb, nc);   // begins and ends with a barrier
  }
  // ynew = W [yu; y_next]
  if (!PF) stage(SW, n + 1, W + (size_t)b * n * n, n, n);
  __syncthreads();
  mv(SW, n + 1, 0, n, nu, yu, cpb, ynew, cpb, nc, T(1), false);
  // the two products split their dot products differently (lengths nu and
  // k), so an output element is finished by a different lane: barrier
  __syncthreads();
  mv(SW, n + 1, nu, n, k, yn, cpb, ynew, cpb, nc, T(1), true);
  __syncthreads();
  if (leaf) {  // leaf level: scatter the solution to the caller's ordering
    scatter(B, ldb, perm, (long long)b * n, ynew, cpb, n, c0, nc);
    return;
  }
  // vnew = U v + D ynew
  if (!PF) {
    stage(SU, k + 1, U + (size_t)b * n * k, n, k);
    __syncthreads();
  }
  mv(SU, k + 1, 0, n, k, vb, cpb, vt, cpb, nc, T(1), false);
  __syncthreads();
  if (!PF) {
    stage(SD, n + 1, D + (size_t)b * n * n, n, n);
    __syncthreads();
  }
  mv(SD, n + 1, 0, n, n, ynew, cpb, vt, cpb, nc, T(1), true);
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    const int i = e / nc, cc = e - i * nc;
    Yout[((size_t)b * n + i) * c + c0 + cc] = ynew[i * cpb + cc];
    Vout[((size_t)b * n + i) * c + c0 + cc] = vt[i * cpb + cc];
  }
}

// Shared-memory elements of the three bodies (see the layouts above).
__host__ __device__ inline size_t ulv_fwd_smem(int n, int cpb) {
  return (size_t)n * (n + 1) + 2 * (size_t)n * cpb;
}
__host__ __device__ inline size_t ulv_root_smem(int n, int cpb, bool pf) {
  return (pf ? 3 : 1) * (size_t)n * (n + 1) + 2 * (size_t)n * cpb;
}
__host__ __device__ inline size_t ulv_bwd_smem(int n, int nu, int k, int cpb, bool pf, bool leaf) {
  const size_t vec = (2 * (size_t)k + nu + 2 * (size_t)n) * cpb;
  if (!pf) return (size_t)n * (n + 1) + vec;
  size_t m = (size_t)nu * (k + 1) + (size_t)nu * (n + 1) + (size_t)n * (n + 1);
  if (!leaf) m += (size_t)n * (k + 1) + (size_t)n * (n + 1);
  return m + vec;
}

}  // namespace ulvk
}  // namespace slu
