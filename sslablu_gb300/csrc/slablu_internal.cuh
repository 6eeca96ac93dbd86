// Internal declarations shared by the slablu translation units.
//
// Storage convention: every matrix is row-major, element (i, j) of a matrix
// with leading dimension ld lives at p[i * ld + j].  HBS levels use the
// stacked "reduced block-diagonal" layout: a level with Nb blocks of n rows and
// c columns is one (Nb*n) x c row-major array, block b starting at row b*n.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <atomic>
#include <map>
#include <memory>
#include <vector>
#include <stdexcept>

#include "../../include/slablu.h"

namespace slu {

// ---------------------------------------------------------------- errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// status codes: SLU_OK / SLU_ERR_* from include/slablu.h

#define SLU_CHECK_CUDA(call)                                                   \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      throw ::slu::Error(SLU_ERR_CUDA,                                  \
                         std::string(#call) + ": " + cudaGetErrorString(e_));  \
  } while (0)

#define SLU_REQUIRE(cond, msg)                                                 \
  do {                                                                         \
    if (!(cond)) throw ::slu::Error(SLU_ERR_ARG, msg);                  \
  } while (0)

// Number of kernels this library has launched (host-side count; reported by
// slu_launch_count so benchmarks can state how many of their kernels ran).
// launch_total() is process wide; launch_thread() is the calling thread's
// share, used to discount launches recorded into a CUDA graph capture.
std::atomic<long long>& launch_total();
long long& launch_thread();
inline void count_launches(long long n) {
  launch_total() += n;
  launch_thread() += n;
}

inline void check_launch(const char* what) {
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    throw Error(SLU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------- memory
// Device buffer owned by the library (stream-ordered allocation).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; bytes = o.bytes; st = o.st;
      o.p = nullptr; o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t b, cudaStream_t s) {
    release();
    st = s;
    bytes = b;
    if (b == 0) return;
    cudaError_t e = cudaMallocAsync(&p, b, s);
    if (e != cudaSuccess) {
      p = nullptr; bytes = 0;
      throw Error(SLU_ERR_ALLOC, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    }
  }
  void release() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    bytes = 0;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// ---------------------------------------------------------------- kernels
// Batched GEMM: for b1 < batch1, b0 < batch0:
//   C_b = alpha * op(A_b) * op(B_b) + beta * C_b,   op(X) = X or X^T
// with X_b = X + b0*sX0 + b1*sX1.  op(A) is M x K, op(B) is K x N.
// beta == 0 never reads C.
template <typename T>
void gemm_batched(cudaStream_t st, bool ta, bool tb, int M, int N, int K, T alpha,
                  const T* A, int lda, long long sA0, long long sA1,
                  const T* B, int ldb, long long sB0, long long sB1, T beta,
                  T* C, int ldc, long long sC0, long long sC1, int batch0, int batch1 = 1);

// Column-major panel QR (LAPACK geqrf convention, v[0] = 1 implicit):
// W_b is an m x ncol column-major array (column j at W_b + j*ldw, contiguous);
// its first nfac columns are factored in place (R on/above the diagonal,
// reflectors below), tau_b[j] the scalar factors; the Householder reflectors
// are applied to all remaining columns nfac..ncol-1 (which then hold Q^T c).
void panel_qr(cudaStream_t st, int m, int nfac, int ncol, double* W, int ldw,
              long long sW, double* tau, long long sTau, int batch);

// The same factorisation for wide panels (nfac > 64): 32-column panels by
// panel_qr, the trailing columns updated in the compact WY form
// (C <- (I - V T^T V^T) C) by three batched GEMMs per panel over all SMs.
// ws holds qr_blocked_ws_elems(m, ncol, batch) doubles; nfac <= 64 runs
// panel_qr itself (ws unused).
size_t qr_blocked_ws_elems(int m, int ncol, int batch);
void qr_blocked(cudaStream_t st, int m, int nfac, int ncol, double* W, int ldw, long long sW,
                double* tau, long long sTau, int batch, double* ws);

// Two panel factorisations of the same shapes in one launch (W, tau and
// W2, tau2, batch blocks each).
void panel_qr2(cudaStream_t st, int m, int nfac, int ncol, double* W, double* W2, int ldw,
               long long sW, double* tau, double* tau2, long long sTau, int batch);

// Apply the reflectors of a factored panel (m x k, column-major, ldv) to the
// columns of C (m x nc, column-major, ldc): C <- Q C (left = false means
// Q^T C).  Used to form Q explicitly from the identity.
void apply_q(cudaStream_t st, bool transpose, int m, int k, const double* V, int ldv,
             long long sV, const double* tau, long long sTau, double* C, int ldc,
             long long sC, int nc, int batch);

// One-sided Jacobi SVD of A_b (m x n, row-major with leading dimension lda):
// writes the leading r left singular vectors (sorted by decreasing singular
// value) as an m x r row-major array U_b (ldu), and the singular values.
// `lower` reads only the lower triangle of A (the rest taken as zero).
void jacobi_left_sv(cudaStream_t st, int m, int n, const double* A, int lda, long long sA,
                    int r, double* U, int ldu, long long sU, double* sv, long long sS,
                    int batch, int* info, bool lower = false);

// Two Jacobi SVDs of the same shapes in one launch (A -> U and A2 -> U2,
// batch blocks each; no singular values).
void jacobi_left_sv2(cudaStream_t st, int m, int n, const double* A, const double* A2, int lda,
                     long long sA, int r, double* U, double* U2, int ldu, long long sU, int batch,
                     int* info, bool lower = false);

// Batched triangular solve with an upper-triangular R_b (n x n): element
// (i, j) of R_b at R_b[i*rRs + j*rCs] (row-major: rRs = ld, rCs = 1;
// column-major: rRs = 1, rCs = ld).  X <- R^{-1} X (trans = false) or
// R^{-T} X where X_b is n x nrhs with element (i, c) at X_b[i*xRs + c*xCs].
template <typename T>
void trsm_upper(cudaStream_t st, bool trans, int n, const T* R, long long rRs, long long rCs,
                long long sR, T* X, long long xRs, long long xCs, long long sX, int nrhs,
                int batch);

// Batched LU with partial pivoting, in place (A_b n x n row-major), pivots
// piv_b[i] = row swapped with row i (LAPACK getrf convention, 0-based).
void lu_factor(cudaStream_t st, int n, double* A, int lda, long long sA, int* piv,
               long long sP, int batch, int* info);
// X <- A^{-1} X (trans=false) or A^{-T} X using the LU factors; X_b n x nrhs row-major.
template <typename T>
void lu_solve(cudaStream_t st, bool trans, int n, const T* LU, int lda, long long sA,
              const int* piv, long long sP, T* X, int ldx, long long sX, int nrhs, int batch);

// Elementwise helpers.
template <typename T>
void axpby(cudaStream_t st, long long n, T a, const T* x, T b, T* y);  // y = a x + b y
void cast_f64_f32(cudaStream_t st, long long n, const double* x, float* y);
void cast_f32_f64(cudaStream_t st, long long n, const float* x, double* y);
void copy2d(cudaStream_t st, int rows, int cols, const double* src, int lds, double* dst,
            int ldd);

// Layout helpers (2-level batches as in gemm_batched).
// dst_b[j*ldd + i] = src_b[i*lds + j] for an rows x cols source.
void transpose_batched(cudaStream_t st, int rows, int cols, const double* src, int lds,
                       long long sS0, long long sS1, double* dst, int ldd, long long sD0,
                       long long sD1, int batch0, int batch1 = 1);
// C_b += alpha * A_b over rows x cols.
template <typename T>
void add_batched(cudaStream_t st, int rows, int cols, T alpha, const T* A, int lda,
                 long long sA0, long long sA1, T* C, int ldc, long long sC0, long long sC1,
                 int batch0, int batch1 = 1);
// C_b = alpha * A_b over rows x cols (plain batched copy when alpha = 1).
template <typename T>
void copy_batched(cudaStream_t st, int rows, int cols, const T* A, int lda, long long sA0,
                  long long sA1, T* C, int ldc, long long sC0, long long sC1, int batch0,
                  int batch1 = 1);
// C_b = identity columns c0..c0+nc-1 of I_m, stored column-major (m x nc, ld m).
void identity_cols(cudaStream_t st, int m, int c0, int nc, double* C, long long sC, int batch);
// dst_b (row-major, ldd) = rows r0..r0+nr-1, columns c0..c0+nc-1 of the upper
// triangle of the column-major array src_b (ld lds); entries below the
// diagonal are written as zero.
void extract_upper(cudaStream_t st, int r0, int nr, int c0, int nc, const double* src, int lds,
                   long long sS, double* dst, int ldd, long long sD, int batch);
void copy_blocks(cudaStream_t st, int nblk, long long width, const void* src, long long spitch,
                 void* dst, long long dpitch);  // bytes

// Split-BF16x3 tensor-core GEMM (tc_gemm.cu): C = alpha A B + beta C, row-major
// float64 in and out, float32 accumulation; ws of tc_gemm_workspace_bytes.
size_t tc_gemm_workspace_bytes(int M, int N, int K);
void tc_gemm_split3(cudaStream_t st, int M, int N, int K, double alpha, const double* A, int lda,
                    const double* B, int ldb, double beta, double* C, int ldc, void* ws,
                    unsigned int* err);

int num_sms();

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) on the current device only
// when a kernel needs more than that device last gave it; the limit only
// grows, under one lock, so concurrent host threads launching the same kernel
// at different sizes cannot lower it under one another (SmemLimit,
// smem_limit.h).  Safe to call while a stream captures.
void ensure_smem(const void* kernel, size_t bytes);

// Host wait for a stream.  By default a spin (cudaStreamSynchronize: the
// lowest latency for a single caller); on a thread that asked for blocking
// waits (set_blocking_waits) the thread sleeps on a blocking-sync event
// instead, so many worker threads waiting at once leave the host cores to
// the threads that are launching work.
void stream_wait(cudaStream_t st);
void set_blocking_waits(bool on);

}  // namespace slu
