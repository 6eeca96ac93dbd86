// HBS apply Y = A X or A^T X as step kernels (sweep.cuh / sweep_host.cuh).
//
// The recursion of HBSnew.HBSMAT.matmat / rmatmat (matAssembly/HBS/
// HBSnew.py:308-350):
//   upward   VV[t+1]_b = F_b^T VV[t]_b          (F = V for A, U for A^T)
//   root     u = op(D_root) VV[L-1]              (op(D) = D^T for A^T)
//   downward u_b = op(D_b) VV[t]_b + G_b u_parent(b)   (G = U for A, V for A^T)
// Each step is one block product with an operator composed from the stored
// factors on first use (hbs_make_apply): F_b^T for the up steps and
// [op(D_b) | G_b] for the down steps, so a down step is a single product
// over [VV[t]_b; u_parent(b)].  The permutation gather of X and scatter of Y
// are folded into the leaf steps.
//
// The double-float apply (the refinement residual of the mixed path) runs the
// same steps on float32 pairs: X is split into pairs, the steps run in
// double-float arithmetic, Y is rounded back to float64.
#include "hbs.cuh"
#include "sweep_host.cuh"

#include <algorithm>

namespace slu {
namespace {

// out_b (n x (n+k)) = [op(D_b) | G_b]
__global__ void compose_down_kernel(int nb, int n, int k, bool transD, const double* __restrict__ D,
                                    const double* __restrict__ G, double* __restrict__ out) {
  const int w = n + k;
  const long long total = (long long)nb * n * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / ((long long)n * w);
    const int r = (int)(e - b * n * w);
    const int i = r / w, j = r - i * w;
    double v;
    if (j < n) v = transD ? D[(b * n + j) * n + i] : D[(b * n + i) * n + j];
    else v = G[(b * n + i) * k + (j - n)];
    out[e] = v;
  }
}

__global__ void split_pairs_kernel(long long n, const double* __restrict__ x,
                                   dfloat* __restrict__ y) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x)
    y[e] = to_dfloat(x[e]);
}

// Y (rows x c, ld c) <- X (ld ldx) as double-float, and back
__global__ void rows_to_pairs_kernel(int rows, int c, const double* __restrict__ X, int ldx,
                                     dfloat* __restrict__ Y) {
  const long long n = (long long)rows * c;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / c, j = e - i * c;
    Y[e] = to_dfloat(X[i * ldx + j]);
  }
}
__global__ void rows_from_pairs_kernel(int rows, int c, const dfloat* __restrict__ Y,
                                       double* __restrict__ X, int ldx) {
  const long long n = (long long)rows * c;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / c, j = e - i * c;
    X[i * ldx + j] = to_double(Y[e]);
  }
}

int grid_for(long long n) {
  return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8LL * num_sms()));
}

void split_pairs(cudaStream_t st, const DevBuf& src, DevBuf& dst) {
  const long long n = (long long)(src.bytes / 8);
  dst.alloc(8 * n, st);
  if (n == 0) return;
  split_pairs_kernel<<<grid_for(n), 256, 0, st>>>(n, src.as<double>(), dst.as<dfloat>());
  check_launch("split_pairs_kernel");
}

template <typename T>
struct ApplyOps;
template <>
struct ApplyOps<double> {
  static bool ready(const Hbs& H, bool trans) { return H.has_apply[trans ? 1 : 0]; }
  static const double* up(const Level& l, bool trans) {
    return (trans ? l.AupT : l.Aup).as<double>();
  }
  static const double* down(const Level& l, bool trans) {
    return (trans ? l.AdnT : l.Adn).as<double>();
  }
};
template <>
struct ApplyOps<dfloat> {
  static bool ready(const Hbs& H, bool trans) { return H.has_df && !trans; }
  static const dfloat* up(const Level& l, bool) { return l.Aupdf.as<dfloat>(); }
  static const dfloat* down(const Level& l, bool) { return l.Adndf.as<dfloat>(); }
};

}  // namespace

void hbs_make_apply(Handle& h, Hbs& H, bool trans) {
  SLU_REQUIRE(H.has_mats, "HBS factors not loaded");
  cudaStream_t st = h.stream;
  const int L = H.L;
  for (int t = 0; t + 1 < L; ++t) {
    Level& l = H.lv[t];
    SLU_REQUIRE(trans ? l.U.p : l.V.p, "apply needs V factors (loaded without V)");
    SLU_REQUIRE(trans ? l.V.p : l.U.p, "apply needs U and V factors");
    const int n = l.n, k = l.k, Nb = l.Nb;
    DevBuf& up = trans ? l.AupT : l.Aup;
    DevBuf& dn = trans ? l.AdnT : l.Adn;
    up.alloc(8 * (size_t)Nb * k * n, st);
    transpose_batched(st, n, k, (trans ? l.U : l.V).as<double>(), k, (long long)n * k, 0,
                      up.as<double>(), n, (long long)k * n, 0, Nb);
    dn.alloc(8 * (size_t)Nb * n * (n + k), st);
    const long long ne = (long long)Nb * n * (n + k);
    compose_down_kernel<<<grid_for(ne), 256, 0, st>>>(Nb, n, k, trans, l.D.as<double>(),
                                                       (trans ? l.V : l.U).as<double>(),
                                                       dn.as<double>());
    check_launch("compose_down_kernel");
  }
  Level& r = H.lv[L - 1];
  DevBuf& dn = trans ? r.AdnT : r.Adn;
  dn.alloc(8 * (size_t)r.n * r.n, st);
  compose_down_kernel<<<grid_for((long long)r.n * r.n), 256, 0, st>>>(
      1, r.n, 0, trans, r.D.as<double>(), nullptr, dn.as<double>());
  check_launch("compose_down_kernel");
  stream_wait(st);
  H.has_apply[trans ? 1 : 0] = true;
}

size_t hbs_apply_scratch_elems(const Hbs& H, int c) {
  size_t vv = 0;
  for (int t = 0; t + 1 < H.L; ++t) vv += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 63) & ~size_t(63);
  return vv + 2 * (((size_t)H.N * c + 63) & ~size_t(63)) + 64;
}

// Y (N x c, ld ldy) = op(A) X; scratch of hbs_apply_scratch_elems elements.
template <typename T>
void hbs_apply_fused(cudaStream_t st, const Hbs& H, bool trans, const T* X, int ldx, T* Y,
                     int ldy, int c, T* scratch) {
  using A = ApplyOps<T>;
  SLU_REQUIRE(A::ready(H, trans), "apply operators not composed");
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  std::vector<T*> VV(L, nullptr);
  size_t off = 0;
  for (int t = 0; t + 1 < L; ++t) {
    VV[t + 1] = scratch + off;
    off += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 63) & ~size_t(63);
  }
  T* u[2] = {scratch + off, scratch + off + (((size_t)H.N * c + 63) & ~size_t(63))};
  if (L == 1) {
    const Level& r = H.lv[0];
    sweep::launch_step(st, sweep::down_step<T>(r, A::down(r, trans), true, X, ldx, perm, nullptr,
                                               Y, ldy, perm, c),
                       "apply_root_step");
    return;
  }
  for (int t = 0; t + 1 < L; ++t) {
    const Level& l = H.lv[t];
    sweep::launch_step(st, sweep::up_step<T>(l, A::up(l, trans), t == 0 ? X : VV[t],
                                             t == 0 ? ldx : c, t == 0 ? perm : nullptr,
                                             VV[t + 1], c),
                       "apply_up_step");
  }
  const Level& r = H.lv[L - 1];
  sweep::launch_step(st, sweep::down_step<T>(r, A::down(r, trans), true, VV[L - 1], c, nullptr,
                                             nullptr, u[0], c, nullptr, c),
                     "apply_root_step");
  int cur = 0;
  for (int t = L - 2; t >= 0; --t) {
    const Level& l = H.lv[t];
    const bool leaf = t == 0;
    sweep::launch_step(st, sweep::down_step<T>(l, A::down(l, trans), false, leaf ? X : VV[t],
                                               leaf ? ldx : c, leaf ? perm : nullptr, u[cur],
                                               leaf ? Y : u[cur ^ 1], leaf ? ldy : c,
                                               leaf ? perm : nullptr, c),
                       "apply_down_step");
    cur ^= 1;
  }
}
template void hbs_apply_fused<double>(cudaStream_t, const Hbs&, bool, const double*, int, double*,
                                      int, int, double*);
template void hbs_apply_fused<dfloat>(cudaStream_t, const Hbs&, bool, const dfloat*, int, dfloat*,
                                      int, int, dfloat*);

// ---------------------------------------------------------------- double-float
void hbs_make_df(Handle& h, Hbs& H) {
  SLU_REQUIRE(H.has_mats, "HBS factors not loaded");
  H.invalidate_plans();
  if (!H.has_apply[0]) hbs_make_apply(h, H, false);
  for (Level& l : H.lv) {
    if (l.Aup.p) split_pairs(h.stream, l.Aup, l.Aupdf);
    split_pairs(h.stream, l.Adn, l.Adndf);
  }
  H.has_df = true;
}

size_t hbs_apply_df_scratch_bytes(const Hbs& H, int c) {
  const size_t nc = ((size_t)H.N * c + 63) & ~size_t(63);
  return sizeof(dfloat) * (2 * nc + hbs_apply_scratch_elems(H, c)) + 256;
}

// Y (N x c, float64, ld ldy) = A X with double-float arithmetic.
void hbs_apply_df(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch) {
  SLU_REQUIRE(H.has_df, "double-float factors not prepared");
  const size_t nc = ((size_t)H.N * c + 63) & ~size_t(63);
  dfloat* xd = static_cast<dfloat*>(scratch);
  dfloat* yd = xd + nc;
  dfloat* ws = yd + nc;
  const long long n = (long long)H.N * c;
  rows_to_pairs_kernel<<<grid_for(n), 256, 0, st>>>(H.N, c, X, ldx, xd);
  check_launch("rows_to_pairs_kernel");
  hbs_apply_fused<dfloat>(st, H, false, xd, c, yd, c, c, ws);
  rows_from_pairs_kernel<<<grid_for(n), 256, 0, st>>>(H.N, c, yd, Y, ldy);
  check_launch("rows_from_pairs_kernel");
}

}  // namespace slu
