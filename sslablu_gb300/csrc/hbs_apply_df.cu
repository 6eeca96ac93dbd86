// Double-float HBS apply for the refinement residual of the mixed path.
//
// Same recursion as hbs_apply.cu (HBSnew.HBSMAT.matmat, matAssembly/HBS/
// HBSnew.py:308-328), with every float64 factor stored as a pair of float32
// (hi, lo), x = hi + lo exactly to 48 bits, and every multiply-accumulate done
// with error-free transformations on float32 units:
//   product  p = ah*xh exactly as (ph, pl) with one fmaf, plus the cross terms
//   sum      TwoSum of the running (hi, lo) with (ph, pl)
// About 13 float32 operations per term; GB300 runs float32 at ~64x its float64
// rate, so the residual b - A x (accurate to ~1e-14 relative) costs a fraction
// of a float64 apply.  Intermediates between levels stay as (hi, lo) pairs.
#include "df_bodies.cuh"
#include "hbs.cuh"

#include <algorithm>

namespace slu {
namespace {

constexpr int kThreads = 256;

using namespace dfk;

__global__ void __launch_bounds__(kThreads)
df_up_kernel(int n, int k, const float* __restrict__ Fh, const float* __restrict__ Fl,
             const double* __restrict__ X, int ldx, const int64_t* __restrict__ perm,
             const DF* __restrict__ in, DF* __restrict__ out, int c, int cpb) {
  extern __shared__ float smf[];
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  df_up_body(smf, b, c0, nc, n, k, Fh, Fl, X, ldx, perm, in, out, c, cpb);
}

__global__ void __launch_bounds__(kThreads)
df_down_kernel(int n, int k, const float* __restrict__ Gh, const float* __restrict__ Gl,
               const float* __restrict__ Dh, const float* __restrict__ Dl,
               const DF* __restrict__ uin, const DF* __restrict__ vv, const double* __restrict__ X,
               int ldx, const int64_t* __restrict__ perm, DF* __restrict__ out,
               double* __restrict__ Y, int ldy, int c, int cpb) {
  extern __shared__ float smf[];
  const int b = blockIdx.x, c0 = blockIdx.y * cpb, nc = min(cpb, c - c0);
  if (nc <= 0) return;
  df_down_body(smf, b, c0, nc, n, k, Gh, Gl, Dh, Dl, uin, vv, X, ldx, perm, out, Y, ldy, c, cpb);
}

__global__ void split_df_kernel(long long n, const double* __restrict__ x, float* __restrict__ h,
                                float* __restrict__ l) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    DF v = split_d(x[e]);
    h[e] = v.h;
    l[e] = v.l;
  }
}

int chunk_df(int Nb, int c) {
  int cpb = c < 16 ? c : 16;
  while (cpb > 2 && (long long)Nb * ((c + cpb - 1) / cpb) < num_sms()) cpb /= 2;
  return cpb;
}

template <typename K>
void set_smem(K kern, size_t bytes) {
  ensure_smem(reinterpret_cast<const void*>(kern), bytes);
}

void split_buf(cudaStream_t st, const DevBuf& src, DevBuf& hi, DevBuf& lo) {
  const long long n = (long long)(src.bytes / 8);
  hi.alloc(4 * n, st);
  lo.alloc(4 * n, st);
  if (n == 0) return;
  long long g = std::min<long long>((n + 255) / 256, 8LL * num_sms());
  split_df_kernel<<<(int)g, 256, 0, st>>>(n, src.as<double>(), hi.as<float>(), lo.as<float>());
  check_launch("split_df_kernel");
}

}  // namespace

void hbs_make_df(Handle& h, Hbs& H) {
  SLU_REQUIRE(H.has_mats, "HBS factors not loaded");
  H.invalidate_plans();
  for (Level& l : H.lv) {
    split_buf(h.stream, l.U, l.Uh, l.Ul);
    split_buf(h.stream, l.V, l.Vh, l.Vl);
    split_buf(h.stream, l.D, l.Dh, l.Dl);
  }
  H.has_df = true;
}

size_t hbs_apply_df_scratch_bytes(const Hbs& H, int c) {
  size_t vv = 0;
  for (int t = 0; t + 1 < H.L; ++t) vv += (((size_t)H.lv[t].Nb * H.lv[t].k * c + 31) & ~size_t(31));
  return sizeof(DF) * (vv + 2 * (((size_t)H.N * c + 31) & ~size_t(31))) + 256;
}

// Y (N x c, float64, ld ldy) = A X with double-float arithmetic.
void hbs_apply_df(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch) {
  SLU_REQUIRE(H.has_df, "double-float factors not prepared");
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  DF* base = reinterpret_cast<DF*>(scratch);
  std::vector<DF*> VV(L, nullptr);
  size_t off = 0;
  for (int t = 0; t + 1 < L; ++t) {
    VV[t + 1] = base + off;
    off += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 31) & ~size_t(31);
  }
  DF* u[2] = {base + off, base + off + (((size_t)H.N * c + 31) & ~size_t(31))};
  auto down = df_down_kernel;
  if (L == 1) {
    const Level& r = H.lv[0];
    const int cpb = chunk_df(1, c);
    size_t sm = 4 * (2 * (size_t)r.n * (r.n + 1) + 4 * (size_t)r.n * cpb);
    set_smem(down, sm);
    down<<<dim3(1, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        r.n, 0, nullptr, nullptr, r.Dh.as<float>(), r.Dl.as<float>(), nullptr, nullptr, X, ldx,
        perm, nullptr, Y, ldy, c, cpb);
    check_launch("df_down_kernel");
    return;
  }
  for (int t = 0; t + 1 < L; ++t) {
    const Level& l = H.lv[t];
    const int cpb = chunk_df(l.Nb, c);
    size_t sm = 4 * (2 * (size_t)l.n * (l.k + 1) + 2 * (size_t)l.n * cpb);
    auto up = df_up_kernel;
    set_smem(up, sm);
    up<<<dim3(l.Nb, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        l.n, l.k, l.Vh.as<float>(), l.Vl.as<float>(), t == 0 ? X : nullptr, ldx,
        t == 0 ? perm : nullptr, VV[t], VV[t + 1], c, cpb);
    check_launch("df_up_kernel");
  }
  const Level& r = H.lv[L - 1];
  {
    const int cpb = chunk_df(1, c);
    size_t sm = 4 * (2 * (size_t)r.n * (r.n + 1) + 4 * (size_t)r.n * cpb);
    set_smem(down, sm);
    down<<<dim3(1, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        r.n, 0, nullptr, nullptr, r.Dh.as<float>(), r.Dl.as<float>(), nullptr, VV[L - 1],
        nullptr, 0, nullptr, u[0], nullptr, 0, c, cpb);
    check_launch("df_down_kernel");
  }
  int cur = 0;
  for (int t = L - 2; t >= 0; --t) {
    const Level& l = H.lv[t];
    const int cpb = chunk_df(l.Nb, c);
    size_t sm = 4 * (2 * (size_t)l.n * (l.n + 1) + (4 * (size_t)l.n + 2 * (size_t)l.k) * cpb);
    set_smem(down, sm);
    const bool leaf = (t == 0);
    down<<<dim3(l.Nb, (c + cpb - 1) / cpb), kThreads, sm, st>>>(
        l.n, l.k, l.Uh.as<float>(), l.Ul.as<float>(), l.Dh.as<float>(), l.Dl.as<float>(), u[cur],
        leaf ? nullptr : VV[t], leaf ? X : nullptr, ldx, leaf ? perm : nullptr,
        leaf ? nullptr : u[cur ^ 1], leaf ? Y : nullptr, ldy, c, cpb);
    check_launch("df_down_kernel");
    cur ^= 1;
  }
}

}  // namespace slu
