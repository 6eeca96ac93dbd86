// Host side of the step kernels (sweep.cuh): the steps of one operator's
// mode-N solve, and the row-slice / column-chunk plan of a launch that runs
// one or more steps (one operator, or one tree step of a group).
#pragma once

#include <algorithm>
#include <vector>

#include "hbs.cuh"
#include "sweep.cuh"

namespace slu {
namespace sweep {

// Forward step t: [ru; x_parent] = Q_b^T x_b.  The leaf step reads the
// caller's right-hand sides through the tree permutation.
template <typename T>
Step<T> forward_step(const Hbs& H, int t, const T* src, int lds, const int64_t* perm, T* ru,
                     T* dst, int c) {
  const Level& l = H.lv[t];
  Step<T> s{};
  s.S = FacPtr<T>::Qt(l);
  s.sS = (long long)l.n * l.n;
  s.rows = l.n;
  s.w = l.n;
  s.nb = l.Nb;
  s.c = c;
  s.nin = 1;
  s.in_p[0] = src;
  s.in_ld[0] = lds;
  s.in_blk[0] = l.n;
  s.in_rows[0] = l.n;
  s.in_perm = perm;
  s.split = l.nu;
  s.out_p[0] = ru;
  s.out_ld[0] = c;
  s.out_blk[0] = l.nu;
  s.out_p[1] = dst;
  s.out_ld[1] = c;
  s.out_blk[1] = l.k;
  return s;
}

// Root: [y; v] = [R^{-1} Q^T; D R^{-1} Q^T] x; a one-level tree solves in
// place through the permutation.
template <typename T>
Step<T> root_step(const Hbs& H, const T* src, int lds, T* B, int ldb, T* Y, T* V, int c) {
  const int L = H.L;
  const Level& r = H.lv[L - 1];
  Step<T> s{};
  s.S = FacPtr<T>::Sw(r);
  s.rows = L == 1 ? r.n : 2 * r.n;
  s.w = r.n;
  s.nb = 1;
  s.c = c;
  s.nin = 1;
  s.in_p[0] = L == 1 ? B : src;
  s.in_ld[0] = L == 1 ? ldb : lds;
  s.in_rows[0] = r.n;
  s.in_perm = L == 1 ? H.perm.as<int64_t>() : nullptr;
  s.split = r.n;
  if (L == 1) {
    s.out_p[0] = B;
    s.out_ld[0] = ldb;
    s.out_perm = H.perm.as<int64_t>();
  } else {
    s.out_p[0] = Y;
    s.out_ld[0] = c;
    s.out_p[1] = V;
    s.out_ld[1] = c;
  }
  return s;
}

// Largest level (rows) the top operator may start at.
constexpr int kTopRows = 256;

// Levels of the solve chain: the top step stands in for levels top .. root.
inline int chain_levels(const Hbs& H) { return H.top >= 1 ? H.top + 1 : H.L; }

// The top step: [y; v] = Top x for the vector x entering level `top`.
template <typename T>
Step<T> top_step(const Hbs& H, const T* src, int lds, T* Y, T* V, int c) {
  const long long M = (long long)H.lv[H.top].Nb * H.lv[H.top].n;
  Step<T> s{};
  s.S = FacPtr<T>::Top(H);
  s.rows = (int)(2 * M);
  s.w = (int)M;
  s.nb = 1;
  s.c = c;
  s.nin = 1;
  s.in_p[0] = src;
  s.in_ld[0] = lds;
  s.in_rows[0] = (int)M;
  s.split = (int)M;
  s.out_p[0] = Y;
  s.out_ld[0] = c;
  s.out_p[1] = V;
  s.out_ld[1] = c;
  return s;
}

// Backward step t: [y_new; v_new] = [G; H] [ru; v; y_next]; the leaf step
// writes y_new to the caller's rows through the permutation.
template <typename T>
Step<T> backward_step(const Hbs& H, int t, const T* ru, const T* Vin, const T* Yin, T* Yout,
                      T* Vout, T* B, int ldb, int c) {
  const Level& l = H.lv[t];
  const bool leaf = t == 0;
  Step<T> s{};
  s.S = FacPtr<T>::Sw(l);
  s.rows = leaf ? l.n : 2 * l.n;
  s.w = l.nu + 2 * l.k;
  s.sS = (long long)s.rows * s.w;
  s.nb = l.Nb;
  s.c = c;
  s.nin = 3;
  s.in_p[0] = ru;
  s.in_ld[0] = c;
  s.in_blk[0] = l.nu;
  s.in_rows[0] = l.nu;
  s.in_p[1] = Vin;
  s.in_ld[1] = c;
  s.in_blk[1] = l.k;
  s.in_rows[1] = l.k;
  s.in_p[2] = Yin;
  s.in_ld[2] = c;
  s.in_blk[2] = l.k;
  s.in_rows[2] = l.k;
  s.split = l.n;
  s.out_blk[0] = l.n;
  if (leaf) {
    s.out_p[0] = B;
    s.out_ld[0] = ldb;
    s.out_perm = H.perm.as<int64_t>();
  } else {
    s.out_p[0] = Yout;
    s.out_ld[0] = c;
    s.out_p[1] = Vout;
    s.out_ld[1] = c;
    s.out_blk[1] = l.n;
  }
  return s;
}

// ---------------------------------------------------------------- mode T
// The mode-T solve (ULVsparse.py:328-353) is the transpose of the mode-N
// map, so it runs the mode-N steps transposed and in reverse order.  Every
// vector of the mode-N solve has one producer and one consumer, so no
// transposed step accumulates into another's output:
//   backward^T, leaf -> root-1:  [ru'; v'; y'] = [G; H]^T z      (SwT)
//   root^T:                      x' = [R^{-1} Q^T; D R^{-1} Q^T]^T z
//   forward^T, root-1 -> leaf:   x_b' = Q_b [ru'; x_parent']
// A backward^T step writes the [v'; y'] rows of a block as one 2k-row range,
// so a parent reads its children's ranges as one input (SwT's columns are
// ordered to match).  The caller's rows enter and leave through iperm.
template <typename T>
Step<T> backwardT_step(const Hbs& H, int t, const T* src, int lds, const int64_t* perm, T* ru,
                       T* dst, int c) {
  const Level& l = H.lv[t];
  const int cols = t == 0 ? l.n : 2 * l.n;
  Step<T> s{};
  s.S = FacPtr<T>::SwT(l);
  s.rows = l.nu + 2 * l.k;
  s.w = cols;
  s.sS = (long long)s.rows * s.w;
  s.nb = l.Nb;
  s.c = c;
  s.nin = 1;
  s.in_p[0] = src;
  s.in_ld[0] = lds;
  s.in_blk[0] = cols;
  s.in_rows[0] = cols;
  s.in_perm = perm;
  s.split = l.nu;
  s.out_p[0] = ru;
  s.out_ld[0] = c;
  s.out_blk[0] = l.nu;
  s.out_p[1] = dst;
  s.out_ld[1] = c;
  s.out_blk[1] = 2 * l.k;
  return s;
}

template <typename T>
Step<T> rootT_step(const Hbs& H, const T* src, int lds, const int64_t* iperm, T* out, int ldo,
                   const int64_t* operm, int c) {
  const Level& r = H.lv[H.L - 1];
  Step<T> s{};
  s.S = FacPtr<T>::SwT(r);
  s.rows = r.n;
  s.w = H.L == 1 ? r.n : 2 * r.n;
  s.nb = 1;
  s.c = c;
  s.nin = 1;
  s.in_p[0] = src;
  s.in_ld[0] = lds;
  s.in_rows[0] = s.w;
  s.in_perm = iperm;
  s.split = r.n;
  s.out_p[0] = out;
  s.out_ld[0] = ldo;
  s.out_perm = operm;
  return s;
}

template <typename T>
Step<T> forwardT_step(const Hbs& H, int t, const T* ru, const T* xp, T* out, int ldo,
                      const int64_t* operm, int c) {
  const Level& l = H.lv[t];
  Step<T> s{};
  s.S = FacPtr<T>::Q(l);
  s.sS = (long long)l.n * l.n;
  s.rows = l.n;
  s.w = l.n;
  s.nb = l.Nb;
  s.c = c;
  s.nin = 2;
  s.in_p[0] = ru;
  s.in_ld[0] = c;
  s.in_blk[0] = l.nu;
  s.in_rows[0] = l.nu;
  s.in_p[1] = xp;
  s.in_ld[1] = c;
  s.in_blk[1] = l.k;
  s.in_rows[1] = l.k;
  s.split = l.n;
  s.out_p[0] = out;
  s.out_ld[0] = ldo;
  s.out_blk[0] = l.n;
  s.out_perm = operm;
  return s;
}

constexpr int kMaxThreads = 256;
constexpr size_t kStepSmem = 96 * 1024;

// Launch plan of a group of steps run by one launch.
struct LaunchPlan {
  long long ctas = 0;
  int threads = 32;
  size_t smem = 0;
};

// Row slices and column chunks of every step of one launch: common caps
// (rows per slice, columns per chunk) lowered until the launch has about two
// CTAs per SM -- row slices first (they split a block operator without
// duplicating its loads), then column chunks.  An in-place step (output 0 is
// the array input 0 is read from: the root of a one-level tree) keeps whole
// blocks per CTA, so every CTA has read its columns' inputs before it writes
// any of them.  Each step then narrows its own slice / chunk until its CTA
// fits in shared memory.
template <typename T>
LaunchPlan plan_steps(Step<T>* const* steps, int count, const PlanKnobs& kn = PlanKnobs()) {
  int rmax = 1, cmax = 1;
  for (int i = 0; i < count; ++i) {
    rmax = std::max(rmax, steps[i]->rows);
    cmax = std::max(cmax, steps[i]->c);
  }
  cmax = std::min(cmax, std::max(1, kn.cmax));
  auto whole = [](const Step<T>* s) { return s->out_p[0] == s->in_p[0]; };
  auto total = [&](int rm, int cm) {
    long long t = 0;
    for (int i = 0; i < count; ++i) {
      const Step<T>* s = steps[i];
      const int rch = whole(s) ? s->rows : std::min(s->rows, rm);
      const int cpb = std::min(s->c, cm);
      t += (long long)s->nb * ((s->rows + rch - 1) / rch) * ((s->c + cpb - 1) / cpb);
    }
    return t;
  };
  const long long target = (long long)std::max(1, kn.target) * num_sms();
  while (total(rmax, cmax) < target) {
    if (rmax > std::max(8, kn.rmin)) rmax = (rmax + 1) / 2;
    else if (cmax > 1) cmax = (cmax + 1) / 2;
    else if (rmax > 8) rmax = (rmax + 1) / 2;
    else break;
  }
  LaunchPlan p;
  for (int i = 0; i < count; ++i) {
    Step<T>& s = *steps[i];
    const bool wh = whole(&s);
    const int ks = split_for<T>(s.w);
    int rch = wh ? s.rows : std::min(s.rows, rmax);
    int cpb = std::min(s.c, cmax);
    auto bytes = [&] { return sizeof(T) * step_smem_elems<T>(rch, s.w, cpb, ks); };
    while (bytes() > kStepSmem) {
      if (rch > 32 && !wh) rch = (rch + 1) / 2;
      else if (cpb > 8) cpb = (cpb + 1) / 2;
      else if (rch > 8 && !wh) rch = (rch + 1) / 2;
      else if (cpb > 1) cpb = (cpb + 1) / 2;
      else break;
    }
    SLU_REQUIRE(bytes() <= kStepSmem, "block operator too wide for the fused ULV solve");
    s.rch = rch;
    s.nrch = (s.rows + rch - 1) / rch;
    s.cpb = cpb;
    const int items = rch * cpb * ks;
    p.threads = std::max(p.threads, std::min(kMaxThreads, (items + 31) / 32 * 32));
    p.smem = std::max(p.smem, bytes());
    p.ctas += (long long)s.nb * s.nrch * ((s.c + cpb - 1) / cpb);
  }
  SLU_REQUIRE(p.ctas < (1LL << 31), "solve step too large");
  return p;
}

// Launch with programmatic stream serialization: the kernel may begin while
// the previous kernel of the stream finishes; step_body waits on it
// (griddepcontrol.wait) before reading anything that kernel writes.
template <typename... Args>
void launch_pdl(void (*kern)(Args...), const LaunchPlan& p, cudaStream_t st,
                const char* what, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)p.ctas);
  cfg.blockDim = dim3((unsigned)p.threads);
  cfg.dynamicSmemBytes = p.smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SLU_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
  check_launch(what);
}

// ---------------------------------------------------------------- apply steps
// The HBS apply Y = op(A) X (HBSnew.HBSMAT.matmat / rmatmat,
// matAssembly/HBS/HBSnew.py:308-350) as the same step kernels:
//   up, level t:   VV[t+1]_b = F_b^T VV[t]_b       S = F_b^T (k x n)
//   root:          u = op(D_root) VV[L-1]           S = op(D_root) (n x n)
//   down, level t: u_b = op(D_b) VV[t]_b + G_b u_parent(b)
//                                                   S = [op(D_b) | G_b] (n x (n+k))
// (F = V, G = U for A; F = U, G = V, op(D) = D^T for A^T).  VV[0] is X read
// through the tree permutation; the leaf down step writes Y through it.
template <typename T>
Step<T> up_step(const Level& l, const T* S, const T* in, int ldi, const int64_t* perm, T* out,
                int c) {
  Step<T> s{};
  s.S = S;
  s.sS = (long long)l.k * l.n;
  s.rows = l.k;
  s.w = l.n;
  s.nb = l.Nb;
  s.c = c;
  s.nin = 1;
  s.in_p[0] = in;
  s.in_ld[0] = ldi;
  s.in_blk[0] = l.n;
  s.in_rows[0] = l.n;
  s.in_perm = perm;
  s.split = l.k;
  s.out_p[0] = out;
  s.out_ld[0] = c;
  s.out_blk[0] = l.k;
  return s;
}

// Down step of level l (root: uin == nullptr, S = op(D) only).
template <typename T>
Step<T> down_step(const Level& l, const T* S, bool root, const T* vv, int ldv,
                  const int64_t* vperm, const T* uin, T* out, int ldo, const int64_t* operm,
                  int c) {
  Step<T> s{};
  s.S = S;
  s.rows = l.n;
  s.w = root ? l.n : l.n + l.k;
  s.sS = (long long)s.rows * s.w;
  s.nb = root ? 1 : l.Nb;
  s.c = c;
  s.nin = root ? 1 : 2;
  s.in_p[0] = vv;
  s.in_ld[0] = ldv;
  s.in_blk[0] = l.n;
  s.in_rows[0] = l.n;
  s.in_perm = vperm;
  if (!root) {
    s.in_p[1] = uin;
    s.in_ld[1] = c;
    s.in_blk[1] = l.k;
    s.in_rows[1] = l.k;
  }
  s.split = l.n;
  s.out_p[0] = out;
  s.out_ld[0] = ldo;
  s.out_blk[0] = l.n;
  s.out_perm = operm;
  return s;
}

// ---------------------------------------------------------------- launches
namespace {
template <typename T>
__global__ void __launch_bounds__(kMaxThreads) step_kernel(const Step<T> s) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int ncch = (s.c + s.cpb - 1) / s.cpb;
  step_body<T>(s, sm_raw, blockIdx.x / ncch, blockIdx.x % ncch);
}
}  // namespace

// Sets the step kernel's shared-memory limit for the plan of `s` (before a
// stream capture, which should contain launches only).
template <typename T>
void prepare_step(Step<T> s, const PlanKnobs& kn = PlanKnobs()) {
  Step<T>* one = &s;
  const LaunchPlan p = plan_steps(&one, 1, kn);
  ensure_smem(reinterpret_cast<const void*>(step_kernel<T>), p.smem);
}

// One step as one launch (programmatic dependent launch); with `lt` the
// launch is bracketed by timing events.
template <typename T>
void launch_step(cudaStream_t st, Step<T> s, const char* what, LaunchTimes* lt = nullptr,
                 int lvl = 0, int kind = 0, const PlanKnobs& kn = PlanKnobs()) {
  Step<T>* one = &s;
  const LaunchPlan p = plan_steps(&one, 1, kn);
  auto kern = step_kernel<T>;
  ensure_smem(reinterpret_cast<const void*>(kern), p.smem);
  if (lt) lt->mark(st);
  launch_pdl(kern, p, st, what, s);
  if (lt) {
    lt->mark(st);
    lt->done(lvl, kind);
  }
}

}  // namespace sweep
}  // namespace slu
