// Dense building blocks: batched GEMM, triangular and LU solves, LU with
// partial pivoting, row permutations and elementwise helpers.
//
// These run the block-diagonal products of the HBS tree levels
// (matAssembly/HBS/HBSnew.py:32-47 block_mult, ULVsparse.py:101-203
// sparse_block_mult / apply_sparse_block), the block solves of the ULV sweep
// (ULVsparse.py:213-226) and the pivot-block LU of the red-black elimination
// (direct_solve/omsdirectsolve.py:211,333 lu_factor / lu_solve).
#include "slablu_internal.cuh"
#include "smem_limit.h"

#include <mutex>
#include <type_traits>

namespace slu {

std::atomic<long long>& launch_total() {
  static std::atomic<long long> n{0};
  return n;
}
long long& launch_thread() {
  static thread_local long long n = 0;
  return n;
}

void ensure_smem(const void* kernel, size_t bytes) {
  static SmemLimit cache;
  int dev = 0;
  SLU_CHECK_CUDA(cudaGetDevice(&dev));
  cudaError_t err = cudaSuccess;
  cache.raise(dev, kernel, bytes, [&](size_t b) {
    err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b);
    return err == cudaSuccess ? 0 : 1;
  });
  if (err != cudaSuccess)
    throw Error(SLU_ERR_CUDA, std::string("cudaFuncSetAttribute(MaxDynamicSharedMemorySize): ") +
                                  cudaGetErrorString(err));
}

namespace {
struct WaitState {
  bool blocking = false;
  int dev = -1;
  cudaEvent_t ev = nullptr;
  ~WaitState() {
    if (ev) cudaEventDestroy(ev);
  }
};
WaitState& wait_state() {
  static thread_local WaitState w;
  return w;
}
}  // namespace

void set_blocking_waits(bool on) { wait_state().blocking = on; }

void stream_wait(cudaStream_t st) {
  WaitState& w = wait_state();
  if (!w.blocking) {
    SLU_CHECK_CUDA(cudaStreamSynchronize(st));
    return;
  }
  int dev = 0;
  SLU_CHECK_CUDA(cudaGetDevice(&dev));
  if (!w.ev || w.dev != dev) {
    if (w.ev) cudaEventDestroy(w.ev);
    w.ev = nullptr;
    SLU_CHECK_CUDA(
        cudaEventCreateWithFlags(&w.ev, cudaEventBlockingSync | cudaEventDisableTiming));
    w.dev = dev;
  }
  SLU_CHECK_CUDA(cudaEventRecord(w.ev, st));
  SLU_CHECK_CUDA(cudaEventSynchronize(w.ev));
}

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

// ============================================================== batched GEMM
// 64x64 output tile per CTA, 256 threads, 4x4 outputs per thread, K step 16.
namespace {
constexpr int GBK = 16;

// TM x TM output tile per CTA (TM = 64, or 32 when 64-tiles would leave most
// SMs idle); 16 x 16 threads, each (TM/16) x (TM/16) outputs.
template <typename T, int TM>
__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, T alpha, const T* __restrict__ A, int lda, long long sA0,
            long long sA1, bool ta, const T* __restrict__ B, int ldb, long long sB0,
            long long sB1, bool tb, T beta, T* __restrict__ C, int ldc, long long sC0,
            long long sC1, int batch0) {
  constexpr int R = TM / 16;
  __shared__ T As[GBK][TM + 1];
  __shared__ T Bs[GBK][TM + 1];
  const int b = blockIdx.z;
  const int b0 = b % batch0, b1 = b / batch0;
  A += b0 * sA0 + b1 * sA1;
  B += b0 * sB0 + b1 * sB1;
  C += b0 * sC0 + b1 * sC1;
  const int row0 = blockIdx.y * TM, col0 = blockIdx.x * TM;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  T acc[R][R];
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int j = 0; j < R; ++j) acc[i][j] = T(0);

  for (int k0 = 0; k0 < K; k0 += GBK) {
#pragma unroll
    for (int e = tid; e < TM * GBK; e += 256) {
      int i, kk;
      if (!ta) { i = e / GBK; kk = e % GBK; } else { kk = e / TM; i = e % TM; }
      int gi = row0 + i, gk = k0 + kk;
      T v = T(0);
      if (gi < M && gk < K) v = ta ? A[(long long)gk * lda + gi] : A[(long long)gi * lda + gk];
      As[kk][i] = v;
    }
#pragma unroll
    for (int e = tid; e < TM * GBK; e += 256) {
      int j, kk;
      if (!tb) { kk = e / TM; j = e % TM; } else { j = e / GBK; kk = e % GBK; }
      int gj = col0 + j, gk = k0 + kk;
      T v = T(0);
      if (gj < N && gk < K) v = tb ? B[(long long)gj * ldb + gk] : B[(long long)gk * ldb + gj];
      Bs[kk][j] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; ++kk) {
      T a[R], bb[R];
#pragma unroll
      for (int i = 0; i < R; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < R; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < R; ++i) {
    int gi = row0 + ty + 16 * i;
    if (gi >= M) continue;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      int gj = col0 + tx + 16 * j;
      if (gj >= N) continue;
      T* c = C + (long long)gi * ldc + gj;
      T v = alpha * acc[i][j];
      if (beta != T(0)) v = fma(beta, *c, v);
      *c = v;
    }
  }
}
// Skinny products (N <= kSkinny columns, B not transposed): the 64 x 64 tile
// kernel would compute 64 output columns per tile regardless of N.  Here each
// output row is one warp (A row-major: lanes stride over K, coalesced, then a
// shuffle reduction per column) or one thread (A transposed: threads over
// rows read A[k][i] coalesced while looping over K); B rows are broadcast.
constexpr int kSkinny = 16;

template <typename T>
__global__ void __launch_bounds__(256)
gemm_skinny_kernel(int M, int N, int K, T alpha, const T* __restrict__ A, int lda,
                   long long sA0, long long sA1, bool ta, const T* __restrict__ B, int ldb,
                   long long sB0, long long sB1, T beta, T* __restrict__ C, int ldc,
                   long long sC0, long long sC1, int batch0) {
  const int b = blockIdx.z;
  const int b0 = b % batch0, b1 = b / batch0;
  A += b0 * sA0 + b1 * sA1;
  B += b0 * sB0 + b1 * sB1;
  C += b0 * sC0 + b1 * sC1;
  T acc[kSkinny];
#pragma unroll
  for (int j = 0; j < kSkinny; ++j) acc[j] = T(0);
  int row;
  if (!ta) {
    const int lane = threadIdx.x & 31;
    row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= M) return;   // whole warp
    const T* a = A + (long long)row * lda;
    for (int k = lane; k < K; k += 32) {
      const T av = a[k];
      const T* bk = B + (long long)k * ldb;
#pragma unroll
      for (int j = 0; j < kSkinny; ++j)
        if (j < N) acc[j] = fma(av, bk[j], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < kSkinny; ++j)
      for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
    if (lane != 0) return;
  } else {
    row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= M) return;
    for (int k = 0; k < K; ++k) {
      const T av = A[(long long)k * lda + row];
      const T* bk = B + (long long)k * ldb;
#pragma unroll
      for (int j = 0; j < kSkinny; ++j)
        if (j < N) acc[j] = fma(av, bk[j], acc[j]);
    }
  }
  T* c = C + (long long)row * ldc;
#pragma unroll
  for (int j = 0; j < kSkinny; ++j)
    if (j < N) {
      T v = alpha * acc[j];
      if (beta != T(0)) v = fma(beta, c[j], v);
      c[j] = v;
    }
}

}  // namespace

template <typename T>
void gemm_batched(cudaStream_t st, bool ta, bool tb, int M, int N, int K, T alpha, const T* A,
                  int lda, long long sA0, long long sA1, const T* B, int ldb, long long sB0,
                  long long sB1, T beta, T* C, int ldc, long long sC0, long long sC1, int batch0,
                  int batch1) {
  if (M <= 0 || N <= 0 || batch0 <= 0 || batch1 <= 0) return;
  if (K <= 0) {  // C = beta C
    SLU_REQUIRE(beta == T(0) || beta == T(1), "gemm with K=0 needs beta 0 or 1");
    if (beta == T(0)) {
      for (int b1 = 0; b1 < batch1; ++b1)
        for (int b0 = 0; b0 < batch0; ++b0)
          SLU_CHECK_CUDA(cudaMemset2DAsync(C + b0 * sC0 + b1 * sC1, sizeof(T) * ldc, 0,
                                           sizeof(T) * N, M, st));
    }
    return;
  }
  long long nb = (long long)batch0 * batch1;
  SLU_REQUIRE(nb <= 65535, "gemm batch too large");
  if (N <= kSkinny && !tb) {
    const int rows_per_cta = ta ? 256 : 8;
    dim3 g((M + rows_per_cta - 1) / rows_per_cta, 1, (unsigned)nb);
    gemm_skinny_kernel<T><<<g, 256, 0, st>>>(M, N, K, alpha, A, lda, sA0, sA1, ta, B, ldb, sB0,
                                             sB1, beta, C, ldc, sC0, sC1, batch0);
    check_launch("gemm_skinny_kernel");
    return;
  }
  const long long tiles64 = (long long)((N + 63) / 64) * ((M + 63) / 64) * nb;
  if (tiles64 < num_sms()) {
    dim3 grid((N + 31) / 32, (M + 31) / 32, (unsigned)nb);
    gemm_kernel<T, 32><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA0, sA1, ta, B, ldb, sB0,
                                             sB1, tb, beta, C, ldc, sC0, sC1, batch0);
  } else {
    dim3 grid((N + 63) / 64, (M + 63) / 64, (unsigned)nb);
    gemm_kernel<T, 64><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA0, sA1, ta, B, ldb, sB0,
                                             sB1, tb, beta, C, ldc, sC0, sC1, batch0);
  }
  check_launch("gemm_kernel");
}

template void gemm_batched<double>(cudaStream_t, bool, bool, int, int, int, double,
                                   const double*, int, long long, long long, const double*, int,
                                   long long, long long, double, double*, int, long long,
                                   long long, int, int);
template void gemm_batched<float>(cudaStream_t, bool, bool, int, int, int, float, const float*,
                                  int, long long, long long, const float*, int, long long,
                                  long long, float, float*, int, long long, long long, int, int);

// ============================================================== triangular solve
// One CTA per (matrix, chunk of right-hand sides).  Column-oriented
// substitution: after x_i is final, every remaining row subtracts R_ri x_i.
namespace {
template <typename T>
__global__ void trsm_upper_kernel(bool trans, int n, const T* __restrict__ R, long long rRs,
                                  long long rCs, long long sR, T* __restrict__ X, long long xRs,
                                  long long xCs, long long sX, int nrhs, int chunk) {
  const int b = blockIdx.y;
  R += b * sR;
  X += b * sX;
  const int c0 = blockIdx.x * chunk;
  const int nc = min(chunk, nrhs - c0);
  if (nc <= 0) return;
  extern __shared__ unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);  // n x nc
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, c = e % nc;
    xs[e] = X[i * xRs + (c0 + c) * xCs];
  }
  __syncthreads();
#define RR(i, j) R[(long long)(i) * rRs + (long long)(j) * rCs]
  if (!trans) {
    for (int i = n - 1; i >= 0; --i) {
      T d = RR(i, i);
      for (int c = threadIdx.x; c < nc; c += blockDim.x) xs[i * nc + c] /= d;
      __syncthreads();
      for (int e = threadIdx.x; e < i * nc; e += blockDim.x) {
        int r = e / nc, c = e % nc;
        xs[e] -= RR(r, i) * xs[i * nc + c];
      }
      __syncthreads();
    }
  } else {
    for (int i = 0; i < n; ++i) {
      T d = RR(i, i);
      for (int c = threadIdx.x; c < nc; c += blockDim.x) xs[i * nc + c] /= d;
      __syncthreads();
      int rem = (n - i - 1) * nc;
      for (int e = threadIdx.x; e < rem; e += blockDim.x) {
        int r = i + 1 + e / nc, c = e % nc;
        xs[r * nc + c] -= RR(i, r) * xs[i * nc + c];
      }
      __syncthreads();
    }
  }
#undef RR
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, c = e % nc;
    X[i * xRs + (c0 + c) * xCs] = xs[e];
  }
}
}  // namespace

template <typename T>
void trsm_upper(cudaStream_t st, bool trans, int n, const T* R, long long rRs, long long rCs,
                long long sR, T* X, long long xRs, long long xCs, long long sX, int nrhs,
                int batch) {
  if (n <= 0 || nrhs <= 0 || batch <= 0) return;
  int chunk = nrhs;
  while ((size_t)n * chunk * sizeof(T) > 96 * 1024 && chunk > 1) chunk = (chunk + 1) / 2;
  while (chunk > 16 && (long long)batch * ((nrhs + chunk - 1) / chunk) < num_sms()) chunk /= 2;
  SLU_REQUIRE((size_t)n * chunk * sizeof(T) <= 96 * 1024, "trsm block too large");
  size_t sm = (size_t)n * chunk * sizeof(T);
  auto kern = trsm_upper_kernel<T>;
  ensure_smem((const void*)kern, sm);
  dim3 grid((nrhs + chunk - 1) / chunk, batch);
  kern<<<grid, 256, sm, st>>>(trans, n, R, rRs, rCs, sR, X, xRs, xCs, sX, nrhs, chunk);
  check_launch("trsm_upper_kernel");
}
template void trsm_upper<double>(cudaStream_t, bool, int, const double*, long long, long long,
                                 long long, double*, long long, long long, long long, int, int);
template void trsm_upper<float>(cudaStream_t, bool, int, const float*, long long, long long,
                                long long, float*, long long, long long, long long, int, int);

// ============================================================== LU (getrf)
namespace {
__device__ inline void argmax_abs_block(double v, int idx, double* sv, int* si, double& out_v,
                                        int& out_i) {
  // warp reduce
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, v, o);
    int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sv[w] = v; si[w] = idx; }
  __syncthreads();
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = lane < nw ? sv[lane] : -1.0;
    idx = lane < nw ? si[lane] : 0x7fffffff;
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, v, o);
      int oi = __shfl_down_sync(0xffffffffu, idx, o);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    if (lane == 0) { sv[0] = v; si[0] = idx; }
  }
  __syncthreads();
  out_v = sv[0];
  out_i = si[0];
  __syncthreads();
}

__global__ void __launch_bounds__(1024)
lu_kernel(int n, double* __restrict__ A, int lda, long long sA, int* __restrict__ piv,
          long long sP, int* info) {
  A += blockIdx.x * sA;
  piv += blockIdx.x * sP;
  __shared__ double sv[32];
  __shared__ int si[32];
  int first_zero = 0;
  for (int j = 0; j < n; ++j) {
    double best = -1.0;
    int bi = j;
    for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
      double v = fabs(A[(long long)i * lda + j]);
      if (v > best) { best = v; bi = i; }
    }
    double pv;
    int p;
    argmax_abs_block(best, bi, sv, si, pv, p);
    if (threadIdx.x == 0) piv[j] = p;
    if (p != j) {
      for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double t = A[(long long)j * lda + c];
        A[(long long)j * lda + c] = A[(long long)p * lda + c];
        A[(long long)p * lda + c] = t;
      }
    }
    __syncthreads();
    double d = A[(long long)j * lda + j];
    if (d == 0.0) {
      if (!first_zero) first_zero = j + 1;
      __syncthreads();
      continue;
    }
    double inv = 1.0 / d;
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) A[(long long)i * lda + j] *= inv;
    __syncthreads();
    int m = n - j - 1;
    for (long long e = threadIdx.x; e < (long long)m * m; e += blockDim.x) {
      int i = j + 1 + (int)(e / m), c = j + 1 + (int)(e % m);
      A[(long long)i * lda + c] -= A[(long long)i * lda + j] * A[(long long)j * lda + c];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && first_zero && info) atomicCAS(info + blockIdx.x, 0, first_zero);
}

// Blocked LU (LAPACK getrf's right-looking scheme): for each panel of kb
// columns, (1) the panel is factored with partial pivoting over all rows
// below its top (one CTA per matrix; the swaps act on the panel's columns),
// (2) the panel's swaps are applied to the other columns and the U row block
// right of the panel is solved with the panel's unit lower triangle, (3) the
// trailing block takes the rank-kb update as one batched GEMM over all SMs.
// The pivots are those of the unblocked elimination (each is chosen in the
// fully updated column).
constexpr int kLuPanel = 32;

__global__ void __launch_bounds__(1024)
lu_panel_kernel(int n, int k0, int kb, double* __restrict__ A, int lda, long long sA,
                int* __restrict__ piv, long long sP, int* info) {
  A += blockIdx.x * sA;
  piv += blockIdx.x * sP;
  __shared__ double sv[32];
  __shared__ int si[32];
  int first_zero = 0;
  const int k1 = k0 + kb;
  for (int j = k0; j < k1; ++j) {
    double best = -1.0;
    int bi = j;
    for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
      const double v = fabs(A[(long long)i * lda + j]);
      if (v > best) { best = v; bi = i; }
    }
    double pv;
    int p;
    argmax_abs_block(best, bi, sv, si, pv, p);
    if (threadIdx.x == 0) piv[j] = p;
    if (p != j) {
      for (int c = k0 + threadIdx.x; c < k1; c += blockDim.x) {
        const double t = A[(long long)j * lda + c];
        A[(long long)j * lda + c] = A[(long long)p * lda + c];
        A[(long long)p * lda + c] = t;
      }
    }
    __syncthreads();
    const double d = A[(long long)j * lda + j];
    if (d == 0.0) {
      if (!first_zero) first_zero = j + 1;
      __syncthreads();
      continue;
    }
    const double inv = 1.0 / d;
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) A[(long long)i * lda + j] *= inv;
    __syncthreads();
    const int w = k1 - j - 1;   // panel columns right of j
    if (w > 0) {
      const long long tot = (long long)(n - j - 1) * w;
      for (long long e = threadIdx.x; e < tot; e += blockDim.x) {
        const int i = j + 1 + (int)(e / w), c = j + 1 + (int)(e % w);
        A[(long long)i * lda + c] -= A[(long long)i * lda + j] * A[(long long)j * lda + c];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && first_zero && info) atomicCAS(info + blockIdx.x, 0, first_zero);
}

// The same panel factorisation with the panel (rows k0.., kb columns) held
// in shared memory, row pitch kb + 1 (column reads hit distinct banks): one
// load, one store, and every column step at shared-memory latency.
constexpr size_t kPanelSmemMax = 200 * 1024;

__global__ void __launch_bounds__(1024)
lu_panel_smem_kernel(int n, int k0, int kb, double* __restrict__ A, int lda, long long sA,
                     int* __restrict__ piv, long long sP, int* info) {
  A += blockIdx.x * sA;
  piv += blockIdx.x * sP;
  extern __shared__ double Ps[];
  __shared__ double sv[32];
  __shared__ int si[32];
  const int R = n - k0, pitch = kb + 1;
  for (int e = threadIdx.x; e < R * kb; e += blockDim.x) {
    const int i = e / kb, c = e - i * kb;
    Ps[i * pitch + c] = A[(long long)(k0 + i) * lda + k0 + c];
  }
  __syncthreads();
  int first_zero = 0;
  for (int jj = 0; jj < kb; ++jj) {
    double best = -1.0;
    int bi = jj;
    for (int i = jj + threadIdx.x; i < R; i += blockDim.x) {
      const double v = fabs(Ps[i * pitch + jj]);
      if (v > best) { best = v; bi = i; }
    }
    double pv;
    int p;
    argmax_abs_block(best, bi, sv, si, pv, p);
    if (threadIdx.x == 0) piv[k0 + jj] = k0 + p;
    if (p != jj) {
      for (int c = threadIdx.x; c < kb; c += blockDim.x) {
        const double t = Ps[jj * pitch + c];
        Ps[jj * pitch + c] = Ps[p * pitch + c];
        Ps[p * pitch + c] = t;
      }
    }
    __syncthreads();
    const double d = Ps[jj * pitch + jj];
    if (d == 0.0) {
      if (!first_zero) first_zero = k0 + jj + 1;
      __syncthreads();
      continue;
    }
    const double inv = 1.0 / d;
    for (int i = jj + 1 + threadIdx.x; i < R; i += blockDim.x) Ps[i * pitch + jj] *= inv;
    __syncthreads();
    const int w = kb - jj - 1;
    if (w > 0) {
      const int tot = (R - jj - 1) * w;
      for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        const int i = jj + 1 + e / w, c = jj + 1 + e % w;
        Ps[i * pitch + c] -= Ps[i * pitch + jj] * Ps[jj * pitch + c];
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < R * kb; e += blockDim.x) {
    const int i = e / kb, c = e - i * kb;
    A[(long long)(k0 + i) * lda + k0 + c] = Ps[i * pitch + c];
  }
  if (threadIdx.x == 0 && first_zero && info) atomicCAS(info + blockIdx.x, 0, first_zero);
}

// One thread per column outside the panel: the panel's row swaps in order,
// then (right of the panel) U12 = L11^{-1} A12 by forward substitution.
__global__ void __launch_bounds__(256)
lu_swap_trsm_kernel(int n, int k0, int kb, double* __restrict__ A, int lda, long long sA,
                    const int* __restrict__ piv, long long sP) {
  A += blockIdx.y * sA;
  piv += blockIdx.y * sP;
  __shared__ double L11[kLuPanel][kLuPanel + 1];
  __shared__ int pv[kLuPanel];
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e / kb, r = e - i * kb;
    L11[i][r] = A[(long long)(k0 + i) * lda + k0 + r];
  }
  for (int j = threadIdx.x; j < kb; j += blockDim.x) pv[j] = piv[k0 + j];
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int k1 = k0 + kb;
  if (c >= n || (c >= k0 && c < k1)) return;
  double* col = A + c;
  for (int j = 0; j < kb; ++j) {
    const int p = pv[j];
    if (p != k0 + j) {
      const double t = col[(long long)(k0 + j) * lda];
      col[(long long)(k0 + j) * lda] = col[(long long)p * lda];
      col[(long long)p * lda] = t;
    }
  }
  if (c < k1) return;
  double x[kLuPanel];
#pragma unroll
  for (int i = 0; i < kLuPanel; ++i) x[i] = i < kb ? col[(long long)(k0 + i) * lda] : 0.0;
#pragma unroll
  for (int i = 1; i < kLuPanel; ++i) {
    double acc = x[i];
#pragma unroll
    for (int r = 0; r < i; ++r) acc -= L11[i][r] * x[r];
    x[i] = acc;
  }
#pragma unroll
  for (int i = 0; i < kLuPanel; ++i)
    if (i < kb) col[(long long)(k0 + i) * lda] = x[i];
}

// Blocked solve with LU factors, for large blocks and many right-hand
// sides (used for the transposed orientation, whose unblocked kernel sweeps
// row by row): the row swaps (one thread per column, in order), then per 32-row
// panel a triangular solve of the panel's rows (one thread per column) and
// the update of the remaining rows as one batched GEMM.
//   mode 0: unit lower L, forward      mode 1: upper U, backward
//   mode 2: U^T (lower), forward       mode 3: unit upper L^T, backward
__global__ void __launch_bounds__(256)
lu_rows_swap_kernel(int n, const int* __restrict__ piv, long long sP, double* __restrict__ X,
                    int ldx, long long sX, int nrhs, bool reverse) {
  piv += blockIdx.y * sP;
  X += blockIdx.y * sX;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  double* col = X + c;
  for (int k = 0; k < n; ++k) {
    const int i = reverse ? n - 1 - k : k;
    const int p = __ldg(piv + i);
    if (p != i) {
      const double t = col[(long long)i * ldx];
      col[(long long)i * ldx] = col[(long long)p * ldx];
      col[(long long)p * ldx] = t;
    }
  }
}

__global__ void __launch_bounds__(256)
lu_panel_solve_kernel(int mode, int k0, int kb, const double* __restrict__ LU, int lda,
                      long long sA, double* __restrict__ X, int ldx, long long sX, int nrhs) {
  LU += blockIdx.y * sA;
  X += blockIdx.y * sX;
  __shared__ double D[kLuPanel][kLuPanel + 1];   // D[i][r]: coefficient of x_r in row i
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e / kb, r = e - i * kb;
    const bool tr = mode >= 2;
    D[i][r] = tr ? LU[(long long)(k0 + r) * lda + k0 + i] : LU[(long long)(k0 + i) * lda + k0 + r];
  }
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  double* col = X + (long long)k0 * ldx + c;
  double x[kLuPanel];
#pragma unroll
  for (int i = 0; i < kLuPanel; ++i) x[i] = i < kb ? col[(long long)i * ldx] : 0.0;
  const bool unit = mode == 0 || mode == 3;
  if (mode == 0 || mode == 2) {   // lower: forward
#pragma unroll
    for (int i = 0; i < kLuPanel; ++i) {
      if (i < kb) {
        double acc = x[i];
#pragma unroll
        for (int r = 0; r < i; ++r) acc -= D[i][r] * x[r];
        x[i] = unit ? acc : acc / D[i][i];
      }
    }
  } else {                        // upper: backward
#pragma unroll
    for (int i = kLuPanel - 1; i >= 0; --i) {
      if (i < kb) {
        double acc = x[i];
#pragma unroll
        for (int r = i + 1; r < kLuPanel; ++r)
          if (r < kb) acc -= D[i][r] * x[r];
        x[i] = unit ? acc : acc / D[i][i];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < kLuPanel; ++i)
    if (i < kb) col[(long long)i * ldx] = x[i];
}

template <typename T>
__global__ void lu_solve_kernel(bool trans, int n, const T* __restrict__ LU, int lda,
                                long long sA, const int* __restrict__ piv, long long sP,
                                T* __restrict__ X, int ldx, long long sX, int nrhs, int chunk) {
  const int b = blockIdx.y;
  LU += b * sA;
  piv += b * sP;
  X += b * sX;
  const int c0 = blockIdx.x * chunk;
  const int nc = min(chunk, nrhs - c0);
  if (nc <= 0) return;
  extern __shared__ unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, c = e % nc;
    xs[e] = X[(long long)i * ldx + c0 + c];
  }
  __syncthreads();
  if (!trans) {
    // P: apply swaps in order
    for (int i = 0; i < n; ++i) {
      int p = piv[i];
      if (p != i)
        for (int c = threadIdx.x; c < nc; c += blockDim.x) {
          T t = xs[i * nc + c]; xs[i * nc + c] = xs[p * nc + c]; xs[p * nc + c] = t;
        }
      __syncthreads();
    }
    // L (unit lower)
    for (int i = 0; i < n; ++i) {
      int rem = (n - i - 1) * nc;
      for (int e = threadIdx.x; e < rem; e += blockDim.x) {
        int r = i + 1 + e / nc, c = e % nc;
        xs[r * nc + c] -= LU[(long long)r * lda + i] * xs[i * nc + c];
      }
      __syncthreads();
    }
    // U
    for (int i = n - 1; i >= 0; --i) {
      T d = LU[(long long)i * lda + i];
      for (int c = threadIdx.x; c < nc; c += blockDim.x) xs[i * nc + c] /= d;
      __syncthreads();
      for (int e = threadIdx.x; e < i * nc; e += blockDim.x) {
        int r = e / nc, c = e % nc;
        xs[e] -= LU[(long long)r * lda + i] * xs[i * nc + c];
      }
      __syncthreads();
    }
  } else {
    // U^T (lower)
    for (int i = 0; i < n; ++i) {
      T d = LU[(long long)i * lda + i];
      for (int c = threadIdx.x; c < nc; c += blockDim.x) xs[i * nc + c] /= d;
      __syncthreads();
      int rem = (n - i - 1) * nc;
      for (int e = threadIdx.x; e < rem; e += blockDim.x) {
        int r = i + 1 + e / nc, c = e % nc;
        xs[r * nc + c] -= LU[(long long)i * lda + r] * xs[i * nc + c];
      }
      __syncthreads();
    }
    // L^T (unit upper)
    for (int i = n - 1; i >= 0; --i) {
      for (int e = threadIdx.x; e < i * nc; e += blockDim.x) {
        int r = e / nc, c = e % nc;
        xs[e] -= LU[(long long)i * lda + r] * xs[i * nc + c];
      }
      __syncthreads();
    }
    // P^T: swaps in reverse order
    for (int i = n - 1; i >= 0; --i) {
      int p = piv[i];
      if (p != i)
        for (int c = threadIdx.x; c < nc; c += blockDim.x) {
          T t = xs[i * nc + c]; xs[i * nc + c] = xs[p * nc + c]; xs[p * nc + c] = t;
        }
      __syncthreads();
    }
  }
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, c = e % nc;
    X[(long long)i * ldx + c0 + c] = xs[e];
  }
}
// X <- A^{-1} X from LAPACK-style LU factors, blocked by 32-row tiles: the
// row swaps are composed into one permutation (one thread) and applied as a
// gather; each diagonal tile is swept by one warp per right-hand-side column
// (lane l holds row l of the tile; the finished x_i is broadcast by shuffle);
// the rows outside the tile are then updated in parallel.  Two block barriers
// per tile instead of one or two per row.  Arithmetic per element as in the
// row-by-row kernel (the same divisions by the pivots).
constexpr int kLuTile = 32;

template <typename T>
__global__ void lu_solve_tiled_kernel(int n, const T* __restrict__ LU, int lda, long long sA,
                                      const int* __restrict__ piv, long long sP,
                                      T* __restrict__ X, int ldx, long long sX, int nrhs,
                                      int chunk) {
  const int b = blockIdx.y;
  LU += b * sA;
  piv += b * sP;
  X += b * sX;
  const int c0 = blockIdx.x * chunk;
  const int nc = min(chunk, nrhs - c0);
  if (nc <= 0) return;
  extern __shared__ unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);                         // n x nc
  T* dt = xs + (size_t)n * nc;                                 // diagonal tile, 32 x 33
  int* perm = reinterpret_cast<int*>(dt + kLuTile * (kLuTile + 1));   // n
  int* pv = perm + n;                                          // n
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = threadIdx.x; i < n; i += blockDim.x) pv[i] = piv[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int i = 0; i < n; ++i) {
      const int p = pv[i];
      const int t = perm[i];
      perm[i] = perm[p];
      perm[p] = t;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    const int i = e / nc, c = e - i * nc;
    xs[e] = X[(long long)perm[i] * ldx + c0 + c];
  }
  // forward: unit lower L
  for (int t0 = 0; t0 < n; t0 += kLuTile) {
    const int tn = min(kLuTile, n - t0);
    for (int e = threadIdx.x; e < tn * tn; e += blockDim.x) {
      const int i = e / tn, j = e - i * tn;
      dt[i * (kLuTile + 1) + j] = LU[(long long)(t0 + i) * lda + t0 + j];
    }
    __syncthreads();
    for (int c = warp; c < nc; c += nw) {
      T xl = lane < tn ? xs[(t0 + lane) * nc + c] : T(0);
      for (int i = 0; i < tn; ++i) {
        const T xi = __shfl_sync(0xffffffffu, xl, i);
        if (lane > i && lane < tn) xl -= dt[lane * (kLuTile + 1) + i] * xi;
      }
      if (lane < tn) xs[(t0 + lane) * nc + c] = xl;
    }
    __syncthreads();
    const int below = n - t0 - tn;
    for (int e = threadIdx.x; e < below * nc; e += blockDim.x) {
      const int r = t0 + tn + e / nc, c = e % nc;
      const T* l = LU + (long long)r * lda + t0;
      T acc = xs[r * nc + c];
      if (tn == kLuTile) {   // full tile: all 32 loads of the row segment in flight
#pragma unroll
        for (int i = 0; i < kLuTile; ++i) acc -= __ldg(l + i) * xs[(t0 + i) * nc + c];
      } else {
        for (int i = 0; i < tn; ++i) acc -= l[i] * xs[(t0 + i) * nc + c];
      }
      xs[r * nc + c] = acc;
    }
    __syncthreads();
  }
  // backward: upper U; each lane inverts its row's pivot up front (all lanes
  // at once) and the sweep multiplies -- a division per row on one lane
  // would serialise the float64 pipe through the whole sweep
  for (int t1 = n; t1 > 0; t1 -= kLuTile) {
    const int t0 = max(0, t1 - kLuTile), tn = t1 - t0;
    for (int e = threadIdx.x; e < tn * tn; e += blockDim.x) {
      const int i = e / tn, j = e - i * tn;
      dt[i * (kLuTile + 1) + j] = LU[(long long)(t0 + i) * lda + t0 + j];
    }
    __syncthreads();
    for (int c = warp; c < nc; c += nw) {
      const T rl = lane < tn ? T(1) / dt[lane * (kLuTile + 1) + lane] : T(0);
      T xl = lane < tn ? xs[(t0 + lane) * nc + c] : T(0);
      for (int i = tn - 1; i >= 0; --i) {
        if (lane == i) xl *= rl;
        const T xi = __shfl_sync(0xffffffffu, xl, i);
        if (lane < i) xl -= dt[lane * (kLuTile + 1) + i] * xi;
      }
      if (lane < tn) xs[(t0 + lane) * nc + c] = xl;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < t0 * nc; e += blockDim.x) {
      const int r = e / nc, c = e % nc;
      const T* u = LU + (long long)r * lda + t0;
      T acc = xs[r * nc + c];
      if (tn == kLuTile) {
#pragma unroll
        for (int i = 0; i < kLuTile; ++i) acc -= __ldg(u + i) * xs[(t0 + i) * nc + c];
      } else {
        for (int i = 0; i < tn; ++i) acc -= u[i] * xs[(t0 + i) * nc + c];
      }
      xs[r * nc + c] = acc;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    const int i = e / nc, c = e - i * nc;
    X[(long long)i * ldx + c0 + c] = xs[e];
  }
}
}  // namespace

void lu_factor(cudaStream_t st, int n, double* A, int lda, long long sA, int* piv, long long sP,
               int batch, int* info) {
  if (n <= 0 || batch <= 0) return;
  if (n <= 2 * kLuPanel) {   // small blocks: one kernel, one CTA per matrix
    lu_kernel<<<batch, 1024, 0, st>>>(n, A, lda, sA, piv, sP, info);
    check_launch("lu_kernel");
    return;
  }
  SLU_REQUIRE(batch <= 65535, "LU batch too large");
  for (int k0 = 0; k0 < n; k0 += kLuPanel) {
    const int kb = std::min(kLuPanel, n - k0), k1 = k0 + kb;
    const size_t psm = sizeof(double) * (size_t)(n - k0) * (kb + 1);
    if (psm <= kPanelSmemMax) {
      ensure_smem(reinterpret_cast<const void*>(lu_panel_smem_kernel), psm);
      lu_panel_smem_kernel<<<batch, 1024, psm, st>>>(n, k0, kb, A, lda, sA, piv, sP, info);
      check_launch("lu_panel_smem_kernel");
    } else {
      lu_panel_kernel<<<batch, 1024, 0, st>>>(n, k0, kb, A, lda, sA, piv, sP, info);
      check_launch("lu_panel_kernel");
    }
    lu_swap_trsm_kernel<<<dim3((n + 255) / 256, batch), 256, 0, st>>>(n, k0, kb, A, lda, sA, piv,
                                                                       sP);
    check_launch("lu_swap_trsm_kernel");
    if (k1 < n)
      gemm_batched<double>(st, false, false, n - k1, n - k1, kb, -1.0,
                           A + (long long)k1 * lda + k0, lda, sA, 0,
                           A + (long long)k0 * lda + k1, lda, sA, 0, 1.0,
                           A + (long long)k1 * lda + k1, lda, sA, 0, batch);
  }
}

namespace {
void lu_solve_blocked(cudaStream_t st, bool trans, int n, const double* LU, int lda, long long sA,
                      const int* piv, long long sP, double* X, int ldx, long long sX, int nrhs,
                      int batch) {
  const dim3 g((nrhs + 255) / 256, batch);
  auto panel = [&](int mode, int k0, int kb) {
    lu_panel_solve_kernel<<<g, 256, 0, st>>>(mode, k0, kb, LU, lda, sA, X, ldx, sX, nrhs);
    check_launch("lu_panel_solve_kernel");
  };
  if (!trans) {
    lu_rows_swap_kernel<<<g, 256, 0, st>>>(n, piv, sP, X, ldx, sX, nrhs, false);
    check_launch("lu_rows_swap_kernel");
    for (int k0 = 0; k0 < n; k0 += kLuPanel) {   // L: rows below -= L21 x1
      const int kb = std::min(kLuPanel, n - k0), k1 = k0 + kb;
      panel(0, k0, kb);
      if (k1 < n)
        gemm_batched<double>(st, false, false, n - k1, nrhs, kb, -1.0,
                             LU + (long long)k1 * lda + k0, lda, sA, 0,
                             X + (long long)k0 * ldx, ldx, sX, 0, 1.0,
                             X + (long long)k1 * ldx, ldx, sX, 0, batch);
    }
    for (int k1 = n; k1 > 0; k1 -= kLuPanel) {   // U: rows above -= U01 x1
      const int k0 = std::max(0, k1 - kLuPanel), kb = k1 - k0;
      panel(1, k0, kb);
      if (k0 > 0)
        gemm_batched<double>(st, false, false, k0, nrhs, kb, -1.0, LU + k0, lda, sA, 0,
                             X + (long long)k0 * ldx, ldx, sX, 0, 1.0, X, ldx, sX, 0, batch);
    }
    return;
  }
  for (int k0 = 0; k0 < n; k0 += kLuPanel) {     // U^T: rows below -= (U12)^T x1
    const int kb = std::min(kLuPanel, n - k0), k1 = k0 + kb;
    panel(2, k0, kb);
    if (k1 < n)
      gemm_batched<double>(st, true, false, n - k1, nrhs, kb, -1.0,
                           LU + (long long)k0 * lda + k1, lda, sA, 0,
                           X + (long long)k0 * ldx, ldx, sX, 0, 1.0,
                           X + (long long)k1 * ldx, ldx, sX, 0, batch);
  }
  for (int k1 = n; k1 > 0; k1 -= kLuPanel) {     // L^T: rows above -= (L10)^T x1
    const int k0 = std::max(0, k1 - kLuPanel), kb = k1 - k0;
    panel(3, k0, kb);
    if (k0 > 0)
      gemm_batched<double>(st, true, false, k0, nrhs, kb, -1.0, LU + (long long)k0 * lda, lda,
                           sA, 0, X + (long long)k0 * ldx, ldx, sX, 0, 1.0, X, ldx, sX, 0,
                           batch);
  }
  lu_rows_swap_kernel<<<g, 256, 0, st>>>(n, piv, sP, X, ldx, sX, nrhs, true);
  check_launch("lu_rows_swap_kernel");
}
}  // namespace

template <typename T>
void lu_solve(cudaStream_t st, bool trans, int n, const T* LU, int lda, long long sA,
              const int* piv, long long sP, T* X, int ldx, long long sX, int nrhs, int batch) {
  if (n <= 0 || nrhs <= 0 || batch <= 0) return;
  if constexpr (std::is_same<T, double>::value) {
    // transposed solves of blocks from 128 with many columns: panels + GEMM
    // updates over all SMs (the tiled one-CTA-per-chunk kernel below serves
    // the other orientation: measured faster there, 163 vs 184 ms in a
    // 1024-point red-black factorisation)
    if (trans && n >= 128 && nrhs >= 64 && batch <= 65535) {
      lu_solve_blocked(st, trans, n, LU, lda, sA, piv, sP, X, ldx, sX, nrhs, batch);
      return;
    }
  }
  int chunk = nrhs;
  while ((size_t)n * chunk * sizeof(T) > 96 * 1024 && chunk > 1) chunk = (chunk + 1) / 2;
  // spread the right-hand sides over ~2 CTAs per SM (the substitutions of
  // different columns are independent)
  while (chunk > (trans ? 16 : 1) && (long long)batch * ((nrhs + chunk - 1) / chunk) < 2 * num_sms())
    chunk = (chunk + 1) / 2;
  size_t sm = (size_t)n * chunk * sizeof(T);
  SLU_REQUIRE(sm <= 96 * 1024, "lu_solve block too large");
  dim3 grid((nrhs + chunk - 1) / chunk, batch);
  if (!trans) {
    auto kern = lu_solve_tiled_kernel<T>;
    const size_t smt = sm + sizeof(T) * kLuTile * (kLuTile + 1) + 2 * sizeof(int) * (size_t)n;
    ensure_smem((const void*)kern, smt);
    kern<<<grid, 256, smt, st>>>(n, LU, lda, sA, piv, sP, X, ldx, sX, nrhs, chunk);
    check_launch("lu_solve_tiled_kernel");
    return;
  }
  auto kern = lu_solve_kernel<T>;
  ensure_smem((const void*)kern, sm);
  kern<<<grid, 256, sm, st>>>(trans, n, LU, lda, sA, piv, sP, X, ldx, sX, nrhs, chunk);
  check_launch("lu_solve_kernel");
}
template void lu_solve<double>(cudaStream_t, bool, int, const double*, int, long long, const int*,
                               long long, double*, int, long long, int, int);
template void lu_solve<float>(cudaStream_t, bool, int, const float*, int, long long, const int*,
                              long long, float*, int, long long, int, int);

// ============================================================== permutations etc.
namespace {
template <typename T>
__global__ void axpby_kernel(long long n, T a, const T* __restrict__ x, T b, T* __restrict__ y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    y[e] = (b == T(0)) ? a * x[e] : fma(a, x[e], b * y[e]);
}
__global__ void cast64_32(long long n, const double* __restrict__ x, float* __restrict__ y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    y[e] = (float)x[e];
}
__global__ void cast32_64(long long n, const float* __restrict__ x, double* __restrict__ y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    y[e] = (double)x[e];
}
inline int grid_for(long long n) {
  long long g = (n + 255) / 256;
  long long cap = 8LL * num_sms();
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}
}  // namespace

template <typename T>
void axpby(cudaStream_t st, long long n, T a, const T* x, T b, T* y) {
  if (n <= 0) return;
  axpby_kernel<T><<<grid_for(n), 256, 0, st>>>(n, a, x, b, y);
  check_launch("axpby_kernel");
}
template void axpby<double>(cudaStream_t, long long, double, const double*, double, double*);
template void axpby<float>(cudaStream_t, long long, float, const float*, float, float*);

void cast_f64_f32(cudaStream_t st, long long n, const double* x, float* y) {
  if (n <= 0) return;
  cast64_32<<<grid_for(n), 256, 0, st>>>(n, x, y);
  check_launch("cast64_32");
}
void cast_f32_f64(cudaStream_t st, long long n, const float* x, double* y) {
  if (n <= 0) return;
  cast32_64<<<grid_for(n), 256, 0, st>>>(n, x, y);
  check_launch("cast32_64");
}
void copy2d(cudaStream_t st, int rows, int cols, const double* src, int lds, double* dst,
            int ldd) {
  if (rows <= 0 || cols <= 0) return;
  SLU_CHECK_CUDA(cudaMemcpy2DAsync(dst, sizeof(double) * ldd, src, sizeof(double) * lds,
                                   sizeof(double) * cols, rows, cudaMemcpyDeviceToDevice, st));
}

// ============================================================== layout helpers
namespace {
__global__ void transpose_kernel(int rows, int cols, const double* __restrict__ src, int lds,
                                 long long sS0, long long sS1, double* __restrict__ dst, int ldd,
                                 long long sD0, long long sD1, int batch0) {
  __shared__ double tile[32][33];
  const int b = blockIdx.z, b0 = b % batch0, b1 = b / batch0;
  src += b0 * sS0 + b1 * sS1;
  dst += b0 * sD0 + b1 * sD1;
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    int i = i0 + r, j = j0 + threadIdx.x;
    if (i < rows && j < cols) tile[r][threadIdx.x] = src[(long long)i * lds + j];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    int j = j0 + r, i = i0 + threadIdx.x;
    if (i < rows && j < cols) dst[(long long)j * ldd + i] = tile[threadIdx.x][r];
  }
}
template <typename T>
__global__ void add_kernel(int rows, int cols, T alpha, const T* __restrict__ A, int lda,
                           long long sA0, long long sA1, T* __restrict__ C, int ldc, long long sC0,
                           long long sC1, int batch0) {
  const int b = blockIdx.y, b0 = b % batch0, b1 = b / batch0;
  A += b0 * sA0 + b1 * sA1;
  C += b0 * sC0 + b1 * sC1;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
    int i = e / cols, j = e % cols;
    C[(long long)i * ldc + j] += alpha * A[(long long)i * lda + j];
  }
}
template <typename T>
__global__ void copyb_kernel(int rows, int cols, const T* __restrict__ A, int lda, long long sA0,
                             long long sA1, T* __restrict__ C, int ldc, long long sC0,
                             long long sC1, int batch0) {
  const int b = blockIdx.y, b0 = b % batch0, b1 = b / batch0;
  A += b0 * sA0 + b1 * sA1;
  C += b0 * sC0 + b1 * sC1;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
    int i = e / cols, j = e % cols;
    C[(long long)i * ldc + j] = A[(long long)i * lda + j];
  }
}
__global__ void identity_cols_kernel(int m, int c0, int nc, double* __restrict__ C, long long sC) {
  C += blockIdx.y * sC;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * nc; e += gridDim.x * blockDim.x) {
    int c = e / m, i = e % m;
    C[e] = (i == c0 + c) ? 1.0 : 0.0;
  }
}
__global__ void extract_upper_kernel(int r0, int nr, int c0, int nc, const double* __restrict__ src,
                                     int lds, long long sS, double* __restrict__ dst, int ldd,
                                     long long sD) {
  src += blockIdx.y * sS;
  dst += blockIdx.y * sD;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nr * nc; e += gridDim.x * blockDim.x) {
    int r = e / nc, c = e % nc;
    int i = r0 + r, j = c0 + c;
    dst[(long long)r * ldd + c] = (i <= j) ? src[(long long)j * lds + i] : 0.0;
  }
}
inline int blocks_for(long long n, int cap) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}
}  // namespace

void transpose_batched(cudaStream_t st, int rows, int cols, const double* src, int lds,
                       long long sS0, long long sS1, double* dst, int ldd, long long sD0,
                       long long sD1, int batch0, int batch1) {
  if (rows <= 0 || cols <= 0 || batch0 <= 0 || batch1 <= 0) return;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32, batch0 * batch1);
  transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(rows, cols, src, lds, sS0, sS1, dst, ldd, sD0,
                                                  sD1, batch0);
  check_launch("transpose_kernel");
}

template <typename T>
void add_batched(cudaStream_t st, int rows, int cols, T alpha, const T* A, int lda, long long sA0,
                 long long sA1, T* C, int ldc, long long sC0, long long sC1, int batch0,
                 int batch1) {
  if (rows <= 0 || cols <= 0 || batch0 <= 0 || batch1 <= 0) return;
  dim3 grid(blocks_for((long long)rows * cols, 64), batch0 * batch1);
  add_kernel<T><<<grid, 256, 0, st>>>(rows, cols, alpha, A, lda, sA0, sA1, C, ldc, sC0, sC1,
                                      batch0);
  check_launch("add_kernel");
}
template void add_batched<double>(cudaStream_t, int, int, double, const double*, int, long long,
                                  long long, double*, int, long long, long long, int, int);
template void add_batched<float>(cudaStream_t, int, int, float, const float*, int, long long,
                                 long long, float*, int, long long, long long, int, int);

template <typename T>
void copy_batched(cudaStream_t st, int rows, int cols, const T* A, int lda, long long sA0,
                  long long sA1, T* C, int ldc, long long sC0, long long sC1, int batch0,
                  int batch1) {
  if (rows <= 0 || cols <= 0 || batch0 <= 0 || batch1 <= 0) return;
  dim3 grid(blocks_for((long long)rows * cols, 64), batch0 * batch1);
  copyb_kernel<T><<<grid, 256, 0, st>>>(rows, cols, A, lda, sA0, sA1, C, ldc, sC0, sC1, batch0);
  check_launch("copyb_kernel");
}
template void copy_batched<double>(cudaStream_t, int, int, const double*, int, long long,
                                   long long, double*, int, long long, long long, int, int);
template void copy_batched<float>(cudaStream_t, int, int, const float*, int, long long, long long,
                                  float*, int, long long, long long, int, int);

void identity_cols(cudaStream_t st, int m, int c0, int nc, double* C, long long sC, int batch) {
  if (m <= 0 || nc <= 0 || batch <= 0) return;
  dim3 grid(blocks_for((long long)m * nc, 64), batch);
  identity_cols_kernel<<<grid, 256, 0, st>>>(m, c0, nc, C, sC);
  check_launch("identity_cols_kernel");
}

void extract_upper(cudaStream_t st, int r0, int nr, int c0, int nc, const double* src, int lds,
                   long long sS, double* dst, int ldd, long long sD, int batch) {
  if (nr <= 0 || nc <= 0 || batch <= 0) return;
  dim3 grid(blocks_for((long long)nr * nc, 64), batch);
  extract_upper_kernel<<<grid, 256, 0, st>>>(r0, nr, c0, nc, src, lds, sS, dst, ldd, sD);
  check_launch("extract_upper_kernel");
}

void copy_blocks(cudaStream_t st, int nblk, long long width, const void* src, long long spitch,
                 void* dst, long long dpitch) {
  if (nblk <= 0 || width <= 0) return;
  SLU_CHECK_CUDA(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, nblk,
                                   cudaMemcpyDeviceToDevice, st));
}

}  // namespace slu
