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
#include "ulv_bodies.cuh"

#include <algorithm>

namespace slu {
namespace {

constexpr int kThreads = 256;
constexpr size_t kSmemPrefetch = 200 * 1024;

using namespace ulvk;

// ---------------------------------------------------------------- per-level kernels
template <typename T>
__global__ void __launch_bounds__(kThreads)
ulv_fwd_kernel(int n, int nu, int k, const T* __restrict__ Q, const T* __restrict__ src, int lds,
               const int64_t* __restrict__ perm, T* __restrict__ ru, T* __restrict__ dst, int c,
               int cpb) {
  extern __shared__ unsigned char sm_raw[];
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  ulv_fwd_body<T>(sm_raw, b, c0, nc, n, nu, k, Q, src, lds, perm, ru, dst, c, cpb);
}

template <typename T, bool PF>
__global__ void __launch_bounds__(kThreads)
ulv_root_kernel(int n, const T* __restrict__ Q, const T* __restrict__ R, const T* __restrict__ D,
                const T* __restrict__ src, int lds, const int64_t* __restrict__ perm,
                T* __restrict__ Yout, T* __restrict__ Vout, T* __restrict__ B, int ldb, int c,
                int cpb) {
  extern __shared__ unsigned char sm_raw[];
  const int c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  ulv_root_body<T, PF>(sm_raw, c0, nc, n, Q, R, D, src, lds, perm, Yout, Vout, B, ldb, c, cpb);
}

template <typename T, bool PF>
__global__ void __launch_bounds__(kThreads)
ulv_bwd_kernel(int n, int nu, int k, const T* __restrict__ ru, const T* __restrict__ Uu,
               const T* __restrict__ R, const T* __restrict__ W, const T* __restrict__ U,
               const T* __restrict__ D, const T* __restrict__ Vin, const T* __restrict__ Yin,
               T* __restrict__ Yout, T* __restrict__ Vout, const int64_t* __restrict__ perm,
               T* __restrict__ B, int ldb, int c, int cpb) {
  extern __shared__ unsigned char sm_raw[];
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  ulv_bwd_body<T, PF>(sm_raw, b, c0, nc, n, nu, k, ru, Uu, R, W, U, D, Vin, Yin, Yout, Vout, perm,
                      B, ldb, c, cpb);
}

// Column chunk per CTA.  float64: the widest chunk that still spreads the
// level over ~2 CTAs per SM (the FP64 pipe bounds the large levels); float32
// (latency bound): chunks of at most 16 columns.
template <typename T>
int chunk_for(int Nb, int c) {
  if (sizeof(T) == 8) {
    const int target = 2 * num_sms();
    int cpb = c;
    while (cpb > 1 && (long long)Nb * ((c + cpb - 1) / cpb) < target) cpb = (cpb + 1) / 2;
    return cpb;
  }
  int cpb = c < 16 ? c : 16;
  while (cpb > 4 && (long long)Nb * ((c + cpb - 1) / cpb) < num_sms()) cpb /= 2;
  return cpb;
}

// Narrows a chunk until its CTA's shared memory (elements of T per column
// `per_col`, fixed part `fixed`) fits in `limit` bytes.
template <typename T>
int fit_chunk(int cpb, size_t fixed, size_t per_col, size_t limit) {
  while (cpb > 1 && sizeof(T) * (fixed + per_col * cpb) > limit) cpb = (cpb + 1) / 2;
  return cpb;
}

template <typename K>
void set_smem(K kern, size_t bytes) {
  ensure_smem(reinterpret_cast<const void*>(kern), bytes);
}

}  // namespace

// B (N x c, caller ordering) <- A^{-1} B; scratch: 5 buffers of stride elements.
template <typename T>
void ulv_solve_fused(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch,
                     size_t stride, LaunchTimes* lt) {
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
    const int cpb = fit_chunk<T>(chunk_for<T>(l.Nb, c), ulv_fwd_smem(l.n, 0), 2 * (size_t)l.n,
                                 kSmemPrefetch);
    size_t sm = sizeof(T) * ulv_fwd_smem(l.n, cpb);
    auto kern = ulv_fwd_kernel<T>;
    set_smem(kern, sm);
    T* dst = P[t & 1];
    dim3 grid(l.Nb, (c + cpb - 1) / cpb);
    if (lt) lt->mark(st);
    kern<<<grid, kThreads, sm, st>>>(l.n, l.nu, l.k, F::Q(l), src, lds, gperm, ru + NN[t] * c,
                                     dst, c, cpb);
    check_launch("ulv_fwd_kernel");
    if (lt) {
      lt->mark(st);
      lt->done(t, 0);
    }
    src = dst;
    lds = c;
    gperm = nullptr;
  }
  // root
  const Level& r = H.lv[L - 1];
  const int cpr = fit_chunk<T>(chunk_for<T>(1, c), ulv_root_smem(r.n, 0, false),
                               2 * (size_t)r.n, kSmemPrefetch);
  {
    // one CTA per column chunk: every block matrix in one asynchronous batch
    // when it fits
    const bool pf = sizeof(T) * ulv_root_smem(r.n, cpr, true) <= kSmemPrefetch;
    size_t sm = sizeof(T) * ulv_root_smem(r.n, cpr, pf);
    auto kern = pf ? ulv_root_kernel<T, true> : ulv_root_kernel<T, false>;
    set_smem(kern, sm);
    dim3 grid(1, (c + cpr - 1) / cpr);
    if (lt) lt->mark(st);
    kern<<<grid, kThreads, sm, st>>>(r.n, F::Q(r), F::R(r), F::D(r), src, lds,
                                     L == 1 ? perm : nullptr, P[2], P[3], B, ldb, c, cpr);
    check_launch("ulv_root_kernel");
    if (lt) {
      lt->mark(st);
      lt->done(L - 1, 1);
    }
  }
  // backward sweep
  int in = 2;
  for (int t = L - 2; t >= 0; --t) {
    const Level& l = H.lv[t];
    const size_t per_col = 2 * (size_t)l.k + l.nu + 2 * (size_t)l.n;
    const int cpb = fit_chunk<T>(chunk_for<T>(l.Nb, c),
                                 ulv_bwd_smem(l.n, l.nu, l.k, 0, false, t == 0), per_col,
                                 kSmemPrefetch);
    dim3 grid(l.Nb, (c + cpb - 1) / cpb);
    // levels that fit in one wave copy all their block matrices in one
    // asynchronous batch (larger shared memory, fewer CTAs per SM)
    const bool leaf = t == 0;
    const bool pf = (long long)grid.x * grid.y <= num_sms() &&
                    sizeof(T) * ulv_bwd_smem(l.n, l.nu, l.k, cpb, true, leaf) <= kSmemPrefetch;
    size_t sm = sizeof(T) * ulv_bwd_smem(l.n, l.nu, l.k, cpb, pf, leaf);
    auto kern = pf ? ulv_bwd_kernel<T, true> : ulv_bwd_kernel<T, false>;
    set_smem(kern, sm);
    const int out = (in == 2) ? 0 : 2;
    if (lt) lt->mark(st);
    kern<<<grid, kThreads, sm, st>>>(l.n, l.nu, l.k, ru + NN[t] * c, F::Uu(l), F::R(l), F::W(l),
                                     F::U(l), F::D(l), P[in + 1], P[in], P[out], P[out + 1],
                                     t == 0 ? perm : nullptr, B, ldb, c, cpb);
    check_launch("ulv_bwd_kernel");
    if (lt) {
      lt->mark(st);
      lt->done(t, 2);
    }
    in = out;
  }
}

namespace {
__global__ void lead_kernel(int us) {
  for (int i = 0; i < us; ++i) __nanosleep(1000);
}
}  // namespace

void enqueue_device_lead(cudaStream_t st, int us) {
  lead_kernel<<<1, 32, 0, st>>>(us);
  check_launch("lead_kernel");
}

template void ulv_solve_fused<double>(cudaStream_t, const Hbs&, double*, int, int, double*, size_t,
                                      LaunchTimes*);
template void ulv_solve_fused<float>(cudaStream_t, const Hbs&, float*, int, int, float*, size_t,
                                     LaunchTimes*);

}  // namespace slu
