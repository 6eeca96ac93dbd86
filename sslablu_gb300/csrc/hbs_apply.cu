// Fused HBS apply: one kernel per tree level and sweep.
//
// u = A v (or A^T v) for the stored HBS factors, the recursion of
// HBSnew.HBSMAT.matmat / rmatmat (matAssembly/HBS/HBSnew.py:308-350):
//   upward   VV[t+1]_b = F_b^T VV[t]_b          (F = V for A, U for A^T)
//   root     u = D_root VV[L-1]                  (D_root^T for A^T)
//   downward u_b = G_b u_parent(b) + D_b VV[t]_b (G = U for A, V for A^T;
//                                                 D_b^T for A^T)
// The permutation gather of v and scatter of u are folded into the leaf
// kernels.  CTA (b, j) handles block b and a chunk of right-hand-side
// columns, staging each block matrix in shared memory (as ulv_solve.cu).
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

// Upward step: out_b (k x c) = F_b^T in_b, in_b n x c (gathered through perm
// on the leaf level).
template <typename T>
__global__ void __launch_bounds__(kThreads)
apply_up_kernel(int n, int k, const T* __restrict__ F, const T* __restrict__ in, int ldi,
                const int64_t* __restrict__ perm, T* __restrict__ out, int c, int cpb) {
  extern __shared__ unsigned char sm_raw[];
  T* S = reinterpret_cast<T*>(sm_raw);   // n x (k+1)
  T* x = S + n * (k + 1);                 // n x cpb
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    long long row = (long long)b * n + i;
    if (perm) row = perm[row];
    x[i * cpb + cc] = in[row * ldi + c0 + cc];
  }
  stage(S, k + 1, F + (size_t)b * n * k, n, k);
  __syncthreads();
  for (int e = threadIdx.x; e < k * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    T acc = T(0);
#pragma unroll 4
    for (int j = 0; j < n; ++j) acc = fma(S[j * (k + 1) + i], x[j * cpb + cc], acc);
    out[((size_t)b * k + i) * c + c0 + cc] = acc;
  }
}

// Downward step (and the root when G == nullptr):
//   out_b = G_b uin_b + op(D_b) vv_b   (n x c); on the leaf level the rows
//   are scattered through perm into Y (ld ldy), and the leaf input vv is
//   gathered through perm from X (ld ldx).
template <typename T>
__global__ void __launch_bounds__(kThreads)
apply_down_kernel(int n, int k, bool transD, const T* __restrict__ G, const T* __restrict__ D,
                  const T* __restrict__ uin, const T* __restrict__ vv, int ldv,
                  const int64_t* __restrict__ perm, T* __restrict__ out, int ldo, int c,
                  int cpb) {
  extern __shared__ unsigned char sm_raw[];
  T* S = reinterpret_cast<T*>(sm_raw);   // n x (n+1)
  T* x = S + n * (n + 1);                 // n x cpb : vv_b
  T* ub = x + n * cpb;                    // k x cpb : uin_b
  T* acc_s = ub + k * cpb;                // n x cpb
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    long long row = (long long)b * n + i;
    if (perm) row = perm[row];
    x[i * cpb + cc] = vv[row * ldv + c0 + cc];
  }
  if (G)
    for (int e = threadIdx.x; e < k * nc; e += blockDim.x) {
      int i = e / nc, cc = e - i * nc;
      ub[i * cpb + cc] = uin[((size_t)b * k + i) * c + c0 + cc];
    }
  stage(S, n + 1, D + (size_t)b * n * n, n, n);
  __syncthreads();
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    T a = T(0);
    if (!transD) {
      const T* s = S + i * (n + 1);
#pragma unroll 4
      for (int j = 0; j < n; ++j) a = fma(s[j], x[j * cpb + cc], a);
    } else {
#pragma unroll 4
      for (int j = 0; j < n; ++j) a = fma(S[j * (n + 1) + i], x[j * cpb + cc], a);
    }
    acc_s[i * cpb + cc] = a;
  }
  if (G) {
    __syncthreads();
    stage(S, k + 1, G + (size_t)b * n * k, n, k);
    __syncthreads();
    for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
      int i = e / nc, cc = e - i * nc;
      const T* s = S + i * (k + 1);
      T a = acc_s[i * cpb + cc];
#pragma unroll 4
      for (int j = 0; j < k; ++j) a = fma(s[j], ub[j * cpb + cc], a);
      acc_s[i * cpb + cc] = a;
    }
  }
  // write (each thread owns its own acc_s entries: no barrier needed)
  for (int e = threadIdx.x; e < n * nc; e += blockDim.x) {
    int i = e / nc, cc = e - i * nc;
    long long row = (long long)b * n + i;
    if (perm) {
      out[perm[row] * ldo + c0 + cc] = acc_s[i * cpb + cc];
    } else {
      out[row * c + c0 + cc] = acc_s[i * cpb + cc];
    }
  }
}

int chunk64(int Nb, int c) {
  int target = 2 * num_sms();
  int cpb = c;
  while (cpb > 1 && (long long)Nb * ((c + cpb - 1) / cpb) < target) cpb = (cpb + 1) / 2;
  return cpb;
}

template <typename K>
void set_smem(K kern, size_t bytes) {
  ensure_smem(reinterpret_cast<const void*>(kern), bytes);
}

}  // namespace

size_t hbs_apply_scratch_elems(const Hbs& H, int c) {
  size_t vv = H.N;
  for (int t = 0; t + 1 < H.L; ++t) vv += (size_t)H.lv[t].Nb * H.lv[t].k;
  return (vv + 2 * (size_t)H.N) * c + 3 * 64;
}

// Y (N x c, ld ldy) = A X or A^T X; scratch of hbs_apply_scratch_elems doubles.
void hbs_apply_fused(cudaStream_t st, const Hbs& H, bool trans, const double* X, int ldx,
                     double* Y, int ldy, int c, double* scratch) {
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  // VV[t] for t >= 1 (VV[0] is X read through perm)
  std::vector<double*> VV(L, nullptr);
  size_t off = 0;
  for (int t = 0; t + 1 < L; ++t) {
    VV[t + 1] = scratch + off;
    off += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 63) & ~size_t(63);
  }
  double* u[2] = {scratch + off, scratch + off + (((size_t)H.N * c + 63) & ~size_t(63))};
  if (L == 1) {
    const Level& r = H.lv[0];
    size_t sm = 8 * ((size_t)r.n * (r.n + 1) + 2 * (size_t)r.n * c);
    auto kern = apply_down_kernel<double>;
    set_smem(kern, sm);
    int cpb = chunk64(1, c);
    sm = 8 * ((size_t)r.n * (r.n + 1) + 2 * (size_t)r.n * cpb);
    set_smem(kern, sm);
    kern<<<dim3(1, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        r.n, 0, trans, nullptr, r.D.as<double>(), nullptr, X, ldx, perm, Y, ldy, c, cpb);
    check_launch("apply_down_kernel");
    return;
  }
  for (int t = 0; t + 1 < L; ++t) {
    const Level& l = H.lv[t];
    const double* F = trans ? l.U.as<double>() : l.V.as<double>();
    const int cpb = chunk64(l.Nb, c);
    size_t sm = 8 * ((size_t)l.n * (l.k + 1) + (size_t)l.n * cpb);
    auto kern = apply_up_kernel<double>;
    set_smem(kern, sm);
    const double* in = t == 0 ? X : VV[t];
    int ldi = t == 0 ? ldx : c;
    kern<<<dim3(l.Nb, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        l.n, l.k, F, in, ldi, t == 0 ? perm : nullptr, VV[t + 1], c, cpb);
    check_launch("apply_up_kernel");
  }
  const Level& r = H.lv[L - 1];
  {
    const int cpb = chunk64(1, c);
    size_t sm = 8 * ((size_t)r.n * (r.n + 1) + 2 * (size_t)r.n * cpb);
    auto kern = apply_down_kernel<double>;
    set_smem(kern, sm);
    kern<<<dim3(1, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        r.n, 0, trans, nullptr, r.D.as<double>(), nullptr, VV[L - 1], c, nullptr, u[0], c, c,
        cpb);
    check_launch("apply_down_kernel");
  }
  int cur = 0;
  for (int t = L - 2; t >= 0; --t) {
    const Level& l = H.lv[t];
    const double* G = trans ? l.V.as<double>() : l.U.as<double>();
    const int cpb = chunk64(l.Nb, c);
    size_t sm = 8 * ((size_t)l.n * (l.n + 1) + (2 * (size_t)l.n + l.k) * cpb);
    auto kern = apply_down_kernel<double>;
    set_smem(kern, sm);
    const bool leaf = (t == 0);
    kern<<<dim3(l.Nb, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        l.n, l.k, trans, G, l.D.as<double>(), u[cur], leaf ? X : VV[t], leaf ? ldx : c,
        leaf ? perm : nullptr, leaf ? Y : u[cur ^ 1], leaf ? ldy : c, c, cpb);
    check_launch("apply_down_kernel");
    cur ^= 1;
  }
}

}  // namespace slu
