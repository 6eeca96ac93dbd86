// Fused ULV solve (mode N): one kernel per tree level and sweep.
//
// Same arithmetic as ULVsparse.solve (matAssembly/HBS/ULVsparse.py:296-327):
//   forward, level t (leaf -> root-1):  z = Q_b^T x_b, the leading nu rows are
//     kept (ru), the trailing k rows form the parent's input;
//   root:  y = R^{-1} (Q^T x),  v = D y;
//   backward, level t (root-1 -> leaf):
//     y_u  = R11^{-1} (ru - Uu v - R12 y_next)
//     ynew = W [y_u; y_next],  vnew = U v + D ynew
//   ynew of the leaf level is the solution (tree order).
// The tree permutation gather (input) and scatter (output) are folded into the
// first and last kernels (HBSnew.py:396-402).
//
// Work split: CTA (b, j) handles block b and a chunk of right-hand-side
// columns; every operation is column independent, so column chunks need no
// communication.  Each CTA stages the block's matrices one at a time in
// shared memory (coalesced, row pitch n+1) and computes from there.  On GB300
// the float64 pipe (~2 DFMA/clk/SM) bounds the f64 sweep, so chunks are sized
// to spread every level over all SMs; the f32 sweep is latency bound and uses
// wider chunks.
//
// Scratch: five N x c buffers (ru, and two ping-pong pairs), the same budget
// as the level-by-level GEMM sweep it replaces.
#include "hbs.cuh"

#include <algorithm>

namespace slu {
namespace {

constexpr int kThreads = 256;

template <typename T>
__device__ inline void stage(T* S, int ld, const T* __restrict__ A, int rows, int cols) {
  for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
    int i = e / cols, j = e - i * cols;
    S[i * ld + j] = A[e];
  }
}

// out[i][c] (+)= sign * sum_j S[i][j0 + j] * x[j][c]   i < rows, j < cols
template <typename T>
__device__ inline void mv(const T* S, int ld, int j0, int rows, int cols, const T* x, int ldx,
                          T* out, int ldo, int nc, T sign, bool accumulate) {
  for (int e = threadIdx.x; e < rows * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    const T* s = S + i * ld + j0;
    T acc = T(0);
#pragma unroll 4
    for (int j = 0; j < cols; ++j) acc = fma(s[j], x[j * ldx + cc], acc);
    T* o = out + i * ldo + cc;
    *o = accumulate ? fma(sign, acc, *o) : sign * acc;
  }
}

// out[i][c] = sum_j S[j][i] * x[j][c]   (transposed product)
template <typename T>
__device__ inline void mvt(const T* S, int ld, int rows_out, int cols_in, const T* x, int ldx,
                           T* out, int ldo, int nc) {
  for (int e = threadIdx.x; e < rows_out * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    T acc = T(0);
#pragma unroll 4
    for (int j = 0; j < cols_in; ++j) acc = fma(S[j * ld + i], x[j * ldx + cc], acc);
    out[i * ldo + cc] = acc;
  }
}

// x <- R^{-1} x for the leading m x m upper triangle of staged R (pitch ld).
template <typename T>
__device__ inline void trsv_upper(const T* R, int ld, int m, T* x, int ldx, int nc) {
  for (int i = m - 1; i >= 0; --i) {
    __syncthreads();
    const T d = R[i * ld + i];
    for (int cc = threadIdx.x; cc < nc; cc += blockDim.x) x[i * ldx + cc] /= d;
    __syncthreads();
    for (int e = threadIdx.x; e < i * nc; e += blockDim.x) {
      int r = e / nc, cc = e - r * nc;
      x[r * ldx + cc] -= R[r * ld + i] * x[i * ldx + cc];
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- forward
template <typename T>
__global__ void __launch_bounds__(kThreads)
ulv_fwd_kernel(int n, int nu, int k, const T* __restrict__ Q, const T* __restrict__ src, int lds,
               const int64_t* __restrict__ perm, T* __restrict__ ru, T* __restrict__ dst, int c,
               int cpb) {
  extern __shared__ unsigned char sm_raw[];
  T* S = reinterpret_cast<T*>(sm_raw);       // n x (n+1)
  T* x = S + n * (n + 1);                     // n x cpb
  T* z = x + n * cpb;                         // n x cpb
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    long long row = (long long)b * n + i;
    if (perm) row = perm[row];
    x[i * cpb + cc] = src[row * lds + c0 + cc];
  }
  stage(S, n + 1, Q + (size_t)b * n * n, n, n);
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
template <typename T>
__global__ void __launch_bounds__(kThreads)
ulv_root_kernel(int n, const T* __restrict__ Q, const T* __restrict__ R, const T* __restrict__ D,
                const T* __restrict__ src, int lds, const int64_t* __restrict__ perm,
                T* __restrict__ Yout, T* __restrict__ Vout, T* __restrict__ B, int ldb, int c,
                int cpb) {
  extern __shared__ unsigned char sm_raw[];
  T* S = reinterpret_cast<T*>(sm_raw);
  T* x = S + n * (n + 1);
  T* y = x + n * cpb;
  const int c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    long long row = perm ? perm[i] : i;
    x[i * cpb + cc] = src[row * lds + c0 + cc];
  }
  stage(S, n + 1, Q, n, n);
  __syncthreads();
  mvt(S, n + 1, n, n, x, cpb, y, cpb, nc);
  __syncthreads();
  stage(S, n + 1, R, n, n);
  trsv_upper(S, n + 1, n, y, cpb, nc);
  if (perm) {  // single-level tree: y is the solution
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
      int i = e / nc, cc = e - i * nc;
      B[perm[i] * ldb + c0 + cc] = y[i * cpb + cc];
    }
    return;
  }
  stage(S, n + 1, D, n, n);
  __syncthreads();
  mv(S, n + 1, 0, n, n, y, cpb, x, cpb, nc, T(1), false);   // x <- D y
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    Yout[(size_t)i * c + c0 + cc] = y[i * cpb + cc];
    Vout[(size_t)i * c + c0 + cc] = x[i * cpb + cc];
  }
}

// ---------------------------------------------------------------- backward
template <typename T>
__global__ void __launch_bounds__(kThreads)
ulv_bwd_kernel(int n, int nu, int k, const T* __restrict__ ru, const T* __restrict__ Uu,
               const T* __restrict__ R, const T* __restrict__ W, const T* __restrict__ U,
               const T* __restrict__ D, const T* __restrict__ Vin, const T* __restrict__ Yin,
               T* __restrict__ Yout, T* __restrict__ Vout, const int64_t* __restrict__ perm,
               T* __restrict__ B, int ldb, int c, int cpb) {
  extern __shared__ unsigned char sm_raw[];
  T* S = reinterpret_cast<T*>(sm_raw);        // n x (n+1) staging
  T* vb = S + n * (n + 1);                     // k  x cpb
  T* yn = vb + k * cpb;                        // k  x cpb
  T* yu = yn + k * cpb;                        // nu x cpb
  T* ynew = yu + nu * cpb;                     // n  x cpb
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  for (int e = threadIdx.x; e < k * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    vb[i * cpb + cc] = Vin[((size_t)b * k + i) * c + c0 + cc];
    yn[i * cpb + cc] = Yin[((size_t)b * k + i) * c + c0 + cc];
  }
  for (int e = threadIdx.x; e < nu * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    yu[i * cpb + cc] = ru[((size_t)b * nu + i) * c + c0 + cc];
  }
  if (nu > 0) {
    // yu = ru - Uu v - R12 y_next ; then R11^{-1}
    stage(S, k + 1, Uu + (size_t)b * nu * k, nu, k);
    __syncthreads();
    mv(S, k + 1, 0, nu, k, vb, cpb, yu, cpb, nc, T(-1), true);
    __syncthreads();
    stage(S, n + 1, R + (size_t)b * nu * n, nu, n);
    __syncthreads();
    mv(S, n + 1, nu, nu, k, yn, cpb, yu, cpb, nc, T(-1), true);
    trsv_upper(S, n + 1, nu, yu, cpb, nc);
  }
  // ynew = W [yu; y_next]
  stage(S, n + 1, W + (size_t)b * n * n, n, n);
  __syncthreads();
  mv(S, n + 1, 0, n, nu, yu, cpb, ynew, cpb, nc, T(1), false);
  mv(S, n + 1, nu, n, k, yn, cpb, ynew, cpb, nc, T(1), true);
  __syncthreads();
  if (perm) {  // leaf level: scatter the solution to the caller's ordering
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
      int i = e / nc, cc = e - i * nc;
      B[perm[(size_t)b * n + i] * ldb + c0 + cc] = ynew[i * cpb + cc];
    }
    return;
  }
  // vnew = U v + D ynew
  T* vn = yu;  // reuse: nu x cpb is too small in general; write straight to Vout below
  (void)vn;
  stage(S, k + 1, U + (size_t)b * n * k, n, k);
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    const T* s = S + i * (k + 1);
    T acc = T(0);
    for (int j = 0; j < k; ++j) acc = fma(s[j], vb[j * cpb + cc], acc);
    Vout[((size_t)b * n + i) * c + c0 + cc] = acc;
    Yout[((size_t)b * n + i) * c + c0 + cc] = ynew[i * cpb + cc];
  }
  __syncthreads();
  stage(S, n + 1, D + (size_t)b * n * n, n, n);
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    const T* s = S + i * (n + 1);
    T acc = T(0);
#pragma unroll 4
    for (int j = 0; j < n; ++j) acc = fma(s[j], ynew[j * cpb + cc], acc);
    Vout[((size_t)b * n + i) * c + c0 + cc] += acc;
  }
}

template <typename T>
int chunk_for(int Nb, int c) {
  if (sizeof(T) == 8) {
    // spread the float64 work over ~2 CTAs per SM
    int target = 2 * num_sms();
    int cpb = c;
    while (cpb > 1 && (long long)Nb * ((c + cpb - 1) / cpb) < target) cpb = (cpb + 1) / 2;
    return cpb;
  }
  int cpb = c < 16 ? c : 16;
  while (cpb > 4 && (long long)Nb * ((c + cpb - 1) / cpb) < num_sms()) cpb /= 2;
  return cpb;
}

template <typename K>
void set_smem(K kern, size_t bytes) {
  ensure_smem(reinterpret_cast<const void*>(kern), bytes);
}

}  // namespace

template <typename T>
struct FacPtr;
template <>
struct FacPtr<double> {
  static const double* U(const Level& l) { return l.U.as<double>(); }
  static const double* D(const Level& l) { return l.D.as<double>(); }
  static const double* Q(const Level& l) { return l.Q.as<double>(); }
  static const double* W(const Level& l) { return l.W.as<double>(); }
  static const double* R(const Level& l) { return l.R.as<double>(); }
  static const double* Uu(const Level& l) { return l.Uu.as<double>(); }
};
template <>
struct FacPtr<float> {
  static const float* U(const Level& l) { return l.Uf.as<float>(); }
  static const float* D(const Level& l) { return l.Df.as<float>(); }
  static const float* Q(const Level& l) { return l.Qf.as<float>(); }
  static const float* W(const Level& l) { return l.Wf.as<float>(); }
  static const float* R(const Level& l) { return l.Rf.as<float>(); }
  static const float* Uu(const Level& l) { return l.Uuf.as<float>(); }
};

// B (N x c, caller ordering) <- A^{-1} B; scratch: 5 buffers of stride elements.
template <typename T>
void ulv_solve_fused(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch,
                     size_t stride) {
  using F = FacPtr<T>;
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  T* ru = scratch;
  T* P[4] = {scratch + stride, scratch + 2 * stride, scratch + 3 * stride, scratch + 4 * stride};
  const std::vector<long long>& NN = H.NN;
  size_t smax = 0;
  for (const Level& l : H.lv) smax = std::max<size_t>(smax, (size_t)l.n * (l.n + 1));
  SLU_REQUIRE(smax * sizeof(T) <= 200 * 1024, "block too large for the fused ULV solve");
  // forward sweep
  const T* src = B;
  int lds = ldb;
  const int64_t* gperm = perm;
  for (int t = 0; t + 1 < L; ++t) {
    const Level& l = H.lv[t];
    const int cpb = chunk_for<T>(l.Nb, c);
    size_t sm = sizeof(T) * ((size_t)l.n * (l.n + 1) + 2 * (size_t)l.n * cpb);
    auto kern = ulv_fwd_kernel<T>;
    set_smem(kern, sm);
    T* dst = P[t & 1];
    dim3 grid(l.Nb, (c + cpb - 1) / cpb);
    kern<<<grid, kThreads, sm, st>>>(l.n, l.nu, l.k, F::Q(l), src, lds, gperm, ru + NN[t] * c,
                                     dst, c, cpb);
    check_launch("ulv_fwd_kernel");
    src = dst;
    lds = c;
    gperm = nullptr;
  }
  // root
  const Level& r = H.lv[L - 1];
  const int cpr = chunk_for<T>(1, c);
  {
    size_t sm = sizeof(T) * ((size_t)r.n * (r.n + 1) + 2 * (size_t)r.n * cpr);
    auto kern = ulv_root_kernel<T>;
    set_smem(kern, sm);
    dim3 grid(1, (c + cpr - 1) / cpr);
    kern<<<grid, kThreads, sm, st>>>(r.n, F::Q(r), F::R(r), F::D(r), src, lds,
                                     L == 1 ? perm : nullptr, P[2], P[3], B, ldb, c, cpr);
    check_launch("ulv_root_kernel");
  }
  // backward sweep
  int in = 2;
  for (int t = L - 2; t >= 0; --t) {
    const Level& l = H.lv[t];
    const int cpb = chunk_for<T>(l.Nb, c);
    size_t sm = sizeof(T) * ((size_t)l.n * (l.n + 1) + (2 * (size_t)l.k + l.nu + l.n) * cpb);
    auto kern = ulv_bwd_kernel<T>;
    set_smem(kern, sm);
    const int out = (in == 2) ? 0 : 2;
    dim3 grid(l.Nb, (c + cpb - 1) / cpb);
    kern<<<grid, kThreads, sm, st>>>(l.n, l.nu, l.k, ru + NN[t] * c, F::Uu(l), F::R(l), F::W(l),
                                     F::U(l), F::D(l), P[in + 1], P[in], P[out], P[out + 1],
                                     t == 0 ? perm : nullptr, B, ldb, c, cpb);
    check_launch("ulv_bwd_kernel");
    in = out;
  }
}

template void ulv_solve_fused<double>(cudaStream_t, const Hbs&, double*, int, int, double*, size_t);
template void ulv_solve_fused<float>(cudaStream_t, const Hbs&, float*, int, int, float*, size_t);

}  // namespace slu
