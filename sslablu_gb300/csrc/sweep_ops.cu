// Composition of the per-block ULV factors into the step operators of the
// mode-N solve (sweep.cuh has the algebra):
//   forward   Qt_b = Q_b^T                                       n x n
//   backward  G_b  = W1 R11^{-1} [I | -Uu | -R12] + [0 | 0 | W2]  n x (nu + 2k)
//             H_b  = D_b G_b + [0 | U_b | 0]     (above the leaves)
//   root      [R^{-1} Q^T ; D R^{-1} Q^T]                         2n x n
// R11^{-1} is applied by the batched triangular solve (back substitution,
// as ULVsparse.solve does per right-hand side, here once per factor column);
// the products are batched float64 GEMMs.
#include "hbs.cuh"
#include "sweep_host.cuh"

#include <algorithm>

namespace slu {
namespace {

// M_b (nu x w, row-major) = [I_nu | -Uu_b | -R12_b]
__global__ void compose_rhs_kernel(int nb, int nu, int k, int n, const double* __restrict__ Uu,
                                   const double* __restrict__ R, double* __restrict__ M) {
  const int w = nu + 2 * k;
  const long long total = (long long)nb * nu * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)nu * w);
    const int r = (int)(e - b * nu * w);
    const int i = r / w, j = r - i * w;
    double v;
    if (j < nu) v = (i == j) ? 1.0 : 0.0;
    else if (j < nu + k) v = -Uu[(b * nu + i) * k + (j - nu)];
    else v = -R[(b * nu + i) * n + nu + (j - nu - k)];
    M[e] = v;
  }
}

__global__ void zero_kernel(long long n, double* __restrict__ x) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    x[e] = 0.0;
}

// ST_b (w x rows) = Sw_b^T with column j taken from row sig(j) of Sw_b:
// sig(j) = j when kc == 0; otherwise j = c*2kc + i runs over child c's
// [v; y] range: i < kc -> v row n + c*kc + i, else y row c*kc + i - kc.
__global__ void transpose_children_kernel(int nb, int rows, int w, int n, int kc,
                                          const double* __restrict__ Sw, double* __restrict__ ST) {
  const long long total = (long long)nb * rows * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)rows * w);
    const int q = (int)(e - b * rows * w);
    const int r = q / rows, j = q - r * rows;
    int src = j;
    if (kc > 0) {
      const int c = j / (2 * kc), i = j - c * 2 * kc;
      src = i < kc ? n + c * kc + i : c * kc + i - kc;
    }
    ST[e] = Sw[(b * rows + src) * w + r];
  }
}

int grid_for(long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8LL * num_sms()));
}

}  // namespace

void hbs_make_sweep(Handle& h, Hbs& H) {
  SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
  cudaStream_t st = h.stream;
  H.invalidate_plans();
  H.tuned.clear();
  ++H.sweep_gen;
  const int L = H.L;
  size_t mmax = 0;
  for (int t = 0; t + 1 < L; ++t) {
    const Level& l = H.lv[t];
    mmax = std::max(mmax, (size_t)l.Nb * l.nu * (l.nu + 2 * (size_t)l.k));
  }
  h.ws.reserve(8 * mmax + 256, st);
  double* M = h.ws.take<double>(std::max<size_t>(mmax, 1));
  for (int t = 0; t + 1 < L; ++t) {
    Level& l = H.lv[t];
    const int n = l.n, k = l.k, nu = l.nu, Nb = l.Nb, w = nu + 2 * k;
    const bool leaf = t == 0;
    const int rows = leaf ? n : 2 * n;
    const long long nn = (long long)n * n, sS = (long long)rows * w;
    l.Qt.alloc(8 * (size_t)Nb * nn, st);
    transpose_batched(st, n, n, l.Q.as<double>(), n, nn, 0, l.Qt.as<double>(), n, nn, 0, Nb);
    l.Sw.alloc(8 * (size_t)Nb * sS, st);
    double* S = l.Sw.as<double>();
    // G = W1 M + [0 | 0 | W2]
    if (nu > 0) {
      const long long ne = (long long)Nb * nu * w;
      compose_rhs_kernel<<<grid_for(ne), 256, 0, st>>>(Nb, nu, k, n, l.Uu.as<double>(),
                                                        l.R.as<double>(), M);
      check_launch("compose_rhs_kernel");
      trsm_upper<double>(st, false, nu, l.R.as<double>(), n, 1, (long long)nu * n, M, w, 1,
                         (long long)nu * w, w, Nb);
      gemm_batched<double>(st, false, false, n, w, nu, 1.0, l.W.as<double>(), n, nn, 0, M, w,
                           (long long)nu * w, 0, 0.0, S, w, sS, 0, Nb);
    } else {
      zero_kernel<<<grid_for((long long)Nb * sS), 256, 0, st>>>((long long)Nb * sS, S);
      check_launch("zero_kernel");
    }
    add_batched<double>(st, n, k, 1.0, l.W.as<double>() + nu, n, nn, 0, S + nu + k, w, sS, 0, Nb);
    if (!leaf) {
      // H = D G + [0 | U | 0]
      gemm_batched<double>(st, false, false, n, w, n, 1.0, l.D.as<double>(), n, nn, 0, S, w, sS,
                           0, 0.0, S + (long long)n * w, w, sS, 0, Nb);
      add_batched<double>(st, n, k, 1.0, l.U.as<double>(), k, (long long)n * k, 0,
                          S + (long long)n * w + nu, w, sS, 0, Nb);
    }
  }
  Level& r = H.lv[L - 1];
  const int n = r.n;
  const long long nn = (long long)n * n;
  r.Sw.alloc(8 * (size_t)(L == 1 ? nn : 2 * nn), st);
  double* S = r.Sw.as<double>();
  transpose_batched(st, n, n, r.Q.as<double>(), n, 0, 0, S, n, 0, 0, 1);
  trsm_upper<double>(st, false, n, r.R.as<double>(), n, 1, 0, S, n, 1, 0, n, 1);
  if (L > 1)
    gemm_batched<double>(st, false, false, n, n, n, 1.0, r.D.as<double>(), n, 0, 0, S, n, 0, 0,
                         0.0, S + nn, n, 0, 0, 1);
  // mode-T operators: every Sw transposed, the columns above the leaves in
  // the order the children's transposed backward steps write [v; y]
  for (int t = 0; t < L; ++t) {
    Level& l = H.lv[t];
    const bool root = t == L - 1;
    const int rows = t == 0 ? l.n : 2 * l.n;
    const int w = root ? l.n : l.nu + 2 * l.k;
    const int nb = root ? 1 : l.Nb;
    const int kc = t == 0 ? 0 : H.lv[t - 1].k;
    SLU_REQUIRE(kc == 0 || l.n % kc == 0, "level size is not a multiple of the children's rank");
    const long long ne = (long long)nb * rows * w;
    l.SwT.alloc(8 * (size_t)ne, st);
    transpose_children_kernel<<<grid_for(ne), 256, 0, st>>>(nb, rows, w, l.n, kc,
                                                            l.Sw.as<double>(), l.SwT.as<double>());
    check_launch("transpose_children_kernel");
  }
  // The top of the mode-N chain as one operator: the steps from the first
  // level of at most kTopRows rows (below the root's children) up to the
  // root and back, applied to the identity, give [y; v] of that level as a
  // 2M x M matrix.  For the C2 tree (M = 256) it holds no more entries than
  // the five steps it replaces.
  H.top = -1;
  H.Top.alloc(0, st);
  int top = -1;
  for (int t = 1; t + 1 < L; ++t)
    if ((long long)H.lv[t].Nb * H.lv[t].n <= sweep::kTopRows) {
      top = t;
      break;
    }
  if (top >= 1) {
    const int M = H.lv[top].Nb * H.lv[top].n;
    const size_t stride = ((size_t)M * M + 31) & ~size_t(31);   // 256-byte aligned
    DevBuf work;
    work.alloc(8 * 6 * stride, st);
    double* I = work.as<double>();
    double* ru = I + stride;
    double* P[4] = {I + 2 * stride, I + 3 * stride, I + 4 * stride, I + 5 * stride};
    identity_cols(st, M, 0, M, I, 0, 1);
    H.Top.alloc(8 * 2 * (size_t)M * M, st);
    double* Tp = H.Top.as<double>();
    const std::vector<long long>& NN = H.NN;
    const double* src = I;
    for (int t = top; t + 1 < L; ++t) {
      sweep::launch_step(st,
                         sweep::forward_step<double>(H, t, src, M, nullptr,
                                                     ru + (NN[t] - NN[top]) * M,
                                                     P[(t - top) & 1], M),
                         "top_compose_step");
      src = P[(t - top) & 1];
    }
    sweep::launch_step(st, sweep::root_step<double>(H, src, M, nullptr, 0, P[2], P[3], M),
                       "top_compose_step");
    int in = 2;
    for (int t = L - 2; t >= top; --t) {
      const int out = in == 2 ? 0 : 2;
      const bool last = t == top;
      sweep::launch_step(st,
                         sweep::backward_step<double>(H, t, ru + (NN[t] - NN[top]) * M, P[in + 1],
                                                      P[in], last ? Tp : P[out],
                                                      last ? Tp + (size_t)M * M : P[out + 1],
                                                      nullptr, 0, M),
                         "top_compose_step");
      in = out;
    }
    H.top = top;
  }
  H.has_sweep = true;
  H.has_f32 = false;
  H.has_dfs = false;
}

}  // namespace slu
