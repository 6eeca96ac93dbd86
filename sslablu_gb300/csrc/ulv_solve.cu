// Fused ULV solve (mode N): one kernel launch per tree level and sweep.
//
// Same result as ULVsparse.solve (matAssembly/HBS/ULVsparse.py:296-327):
//   forward, level t (leaf -> root-1):  z = Q_b^T x_b, the leading nu rows are
//     kept (ru), the trailing k rows form the parent's input;
//   root:  y = R^{-1} (Q^T x),  v = D y;
//   backward, level t (root-1 -> leaf):
//     y_u  = R11^{-1} (ru - Uu v - R12 y_next)
//     ynew = W [y_u; y_next],  vnew = U v + D ynew
//   ynew of the leaf level is the solution (tree order).
// Each step runs as one block-sparse product with the operators composed at
// factor time (sweep.cuh, sweep_ops.cu); the tree permutation gather (input)
// and scatter (output) are folded into the first and last launches
// (HBSnew.py:396-402).
//
// Work split: a CTA computes a slice of output rows of one block for a chunk
// of right-hand-side columns (plan_steps, sweep_host.cuh).
//
// Scratch: five N x c buffers (ru, and two ping-pong pairs).
#include "hbs.cuh"
#include "sweep_host.cuh"

#include <algorithm>

namespace slu {

using sweep::launch_step;

// B (N x c, caller ordering) <- A^{-1} B; scratch: 5 buffers of stride elements.
template <typename T>
void ulv_solve_fused(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch,
                     size_t stride, LaunchTimes* lt) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  T* ru = scratch;
  T* P[4] = {scratch + stride, scratch + 2 * stride, scratch + 3 * stride, scratch + 4 * stride};
  const std::vector<long long>& NN = H.NN;
  const T* src = B;
  int lds = ldb;
  for (int t = 0; t + 1 < L; ++t) {
    launch_step(st, sweep::forward_step<T>(H, t, src, lds, t == 0 ? perm : nullptr,
                                           ru + NN[t] * c, P[t & 1], c),
                "ulv_fwd_step", lt, t, 0);
    src = P[t & 1];
    lds = c;
  }
  launch_step(st, sweep::root_step<T>(H, src, lds, B, ldb, P[2], P[3], c), "ulv_root_step", lt,
              L - 1, 1);
  int in = 2;
  for (int t = L - 2; t >= 0; --t) {
    const int out = (in == 2) ? 0 : 2;
    launch_step(st, sweep::backward_step<T>(H, t, ru + NN[t] * c, P[in + 1], P[in], P[out],
                                            P[out + 1], B, ldb, c),
                "ulv_bwd_step", lt, t, 2);
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
template void ulv_solve_fused<dfloat>(cudaStream_t, const Hbs&, dfloat*, int, int, dfloat*, size_t,
                                      LaunchTimes*);

// ---------------------------------------------------------------- double-float sweep
namespace {
__global__ void split_dfs_kernel(long long n, const double* __restrict__ x,
                                 dfloat* __restrict__ y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    y[e] = to_dfloat(x[e]);
}

// Y (rows x c, ld c) <- X (ld ldx) as double-float, or back
__global__ void rhs_to_dfs_kernel(int rows, int c, const double* __restrict__ X, int ldx,
                                  dfloat* __restrict__ Y) {
  const long long n = (long long)rows * c;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / c, j = e - i * c;
    Y[e] = to_dfloat(X[i * ldx + j]);
  }
}
__global__ void rhs_from_dfs_kernel(int rows, int c, const dfloat* __restrict__ Y,
                                    double* __restrict__ X, int ldx) {
  const long long n = (long long)rows * c;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / c, j = e - i * c;
    X[i * ldx + j] = to_double(Y[e]);
  }
}

int elem_grid(long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8LL * num_sms()));
}

void split_dfs(cudaStream_t st, const DevBuf& src, DevBuf& dst) {
  const long long n = (long long)(src.bytes / 8);
  dst.alloc(8 * n, st);
  if (n == 0) return;
  split_dfs_kernel<<<elem_grid(n), 256, 0, st>>>(n, src.as<double>(), dst.as<dfloat>());
  check_launch("split_dfs_kernel");
}
}  // namespace

void hbs_make_dfs(Handle& h, Hbs& H) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  H.invalidate_plans();
  cudaStream_t st = h.stream;
  for (Level& l : H.lv) {
    split_dfs(st, l.Qt, l.Qtdf);
    split_dfs(st, l.Sw, l.Swdf);
  }
  H.has_dfs = true;
}

size_t hbs_solve_df_scratch_bytes(const Hbs& H, int c) {
  const size_t one = (sizeof(dfloat) * (size_t)H.N * c + 255) & ~size_t(255);
  return 6 * one;
}

void hbs_solve_df(cudaStream_t st, const Hbs& H, double* B, int ldb, int c, void* scratch) {
  SLU_REQUIRE(H.has_dfs, "double-float factors not prepared");
  const size_t stride = ((sizeof(dfloat) * (size_t)H.N * c + 255) & ~size_t(255)) / sizeof(dfloat);
  dfloat* Bd = static_cast<dfloat*>(scratch);
  const long long n = (long long)H.N * c;
  rhs_to_dfs_kernel<<<elem_grid(n), 256, 0, st>>>(H.N, c, B, ldb, Bd);
  check_launch("rhs_to_dfs_kernel");
  ulv_solve_fused<dfloat>(st, H, Bd, c, c, Bd + stride, stride);
  rhs_from_dfs_kernel<<<elem_grid(n), 256, 0, st>>>(H.N, c, Bd, B, ldb);
  check_launch("rhs_from_dfs_kernel");
}

}  // namespace slu
