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
#include <array>

namespace slu {

using sweep::launch_step;

namespace {

template <typename T>
struct StepRec {
  sweep::Step<T> s;
  const char* what;
  int level, kind;
};

template <typename T> constexpr int type_code();
template <> constexpr int type_code<double>() { return 0; }
template <> constexpr int type_code<float>() { return 1; }
template <> constexpr int type_code<dfloat>() { return 2; }

// The launches of a mode-N solve, in order (2L-1, or 2 top + 1 with the top
// levels as one composed operator): the right-hand sides are
// read from X (ld ldx) and the solution written to B (ld ldb); X == B solves
// in place.
template <typename T>
std::vector<StepRec<T>> solve_steps(const Hbs& H, const T* X, int ldx, T* B, int ldb, int c,
                                    T* scratch, size_t stride) {
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  T* ru = scratch;
  T* P[4] = {scratch + stride, scratch + 2 * stride, scratch + 3 * stride, scratch + 4 * stride};
  const std::vector<long long>& NN = H.NN;
  std::vector<StepRec<T>> v;
  const T* src = X;
  int lds = ldx;
  const int Lc = sweep::chain_levels(H);
  for (int t = 0; t + 1 < Lc; ++t) {
    v.push_back({sweep::forward_step<T>(H, t, src, lds, t == 0 ? perm : nullptr, ru + NN[t] * c,
                                        P[t & 1], c),
                 "ulv_fwd_step", t, 0});
    src = P[t & 1];
    lds = c;
  }
  if (H.top >= 1)
    v.push_back({sweep::top_step<T>(H, src, lds, P[2], P[3], c), "ulv_top_step", H.top, 1});
  else
    v.push_back({sweep::root_step<T>(H, src, lds, B, ldb, P[2], P[3], c), "ulv_root_step", L - 1,
                 1});
  if (L == 1 && X != B) {   // one-level tree: the root reads X, writes B
    sweep::Step<T>& r = v.back().s;
    r.in_p[0] = X;
    r.in_ld[0] = ldx;
  }
  int in = 2;
  for (int t = Lc - 2; t >= 0; --t) {
    const int out = (in == 2) ? 0 : 2;
    v.push_back({sweep::backward_step<T>(H, t, ru + NN[t] * c, P[in + 1], P[in], P[out],
                                         P[out + 1], B, ldb, c),
                 "ulv_bwd_step", t, 2});
    in = out;
  }
  return v;
}

// The 2L-1 launches of a mode-T solve (sweep_host.cuh): right-hand sides
// read from X, solution written to B.  Scratch: ru' (one stride, at the
// mode-N offsets) and two ping-pong buffers of two strides each (a
// backward^T step writes 2k rows per block: at most 2N).
template <typename T>
std::vector<StepRec<T>> solve_steps_T(const Hbs& H, const T* X, int ldx, T* B, int ldb, int c,
                                      T* scratch, size_t stride) {
  const int L = H.L;
  const int64_t* ip = H.iperm.as<int64_t>();
  T* ru = scratch;
  T* P[2] = {scratch + stride, scratch + 3 * stride};
  const std::vector<long long>& NN = H.NN;
  std::vector<StepRec<T>> v;
  if (L == 1) {
    v.push_back({sweep::rootT_step<T>(H, X, ldx, ip, B, ldb, ip, c), "ulvT_root_step", 0, 1});
    return v;
  }
  for (int t = 0; t + 1 < L; ++t)
    v.push_back({sweep::backwardT_step<T>(H, t, t == 0 ? X : P[(t - 1) & 1], t == 0 ? ldx : c,
                                          t == 0 ? ip : nullptr, ru + NN[t] * c, P[t & 1], c),
                 "ulvT_bwd_step", t, 2});
  int cur = (L - 1) & 1;
  v.push_back({sweep::rootT_step<T>(H, P[(L - 2) & 1], c, nullptr, P[cur], c, nullptr, c),
               "ulvT_root_step", L - 1, 1});
  for (int t = L - 2; t >= 0; --t) {
    const bool leaf = t == 0;
    v.push_back({sweep::forwardT_step<T>(H, t, ru + NN[t] * c, P[cur], leaf ? B : P[cur ^ 1],
                                         leaf ? ldb : c, leaf ? ip : nullptr, c),
                 "ulvT_fwd_step", t, 0});
    cur ^= 1;
  }
  return v;
}

}  // namespace

// B (N x c, caller ordering) <- A^{-T} B with the transposed steps; X as in
// ulv_solve_fused.
template <typename T>
void ulv_solve_T(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch, size_t stride,
                 const T* X, int ldx) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  if (!X) {
    X = B;
    ldx = ldb;
  }
  for (const StepRec<T>& r : solve_steps_T<T>(H, X, ldx, B, ldb, c, scratch, stride))
    launch_step(st, r.s, r.what);
}
template void ulv_solve_T<double>(cudaStream_t, const Hbs&, double*, int, int, double*, size_t,
                                  const double*, int);
template void ulv_solve_T<float>(cudaStream_t, const Hbs&, float*, int, int, float*, size_t,
                                 const float*, int);

// B (N x c, caller ordering) <- A^{-1} B; scratch: 5 buffers of stride elements.
template <typename T>
void ulv_solve_fused(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch,
                     size_t stride, LaunchTimes* lt, const T* X, int ldx) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  if (!X) {
    X = B;
    ldx = ldb;
  }
  const std::vector<StepRec<T>> steps = solve_steps<T>(H, X, ldx, B, ldb, c, scratch, stride);
  auto it = H.tuned.find({type_code<T>(), c});
  const std::vector<PlanKnobs>* kn =
      (it != H.tuned.end() && it->second.size() == steps.size()) ? &it->second : nullptr;
  for (size_t i = 0; i < steps.size(); ++i)
    launch_step(st, steps[i].s, steps[i].what, lt, steps[i].level, steps[i].kind,
                kn ? (*kn)[i] : PlanKnobs());
}

void solve_plan_create(Handle& h, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                       int c, bool trans, SolvePlan& P) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  cudaStream_t st = h.stream;
  const size_t stride = ((8 * (size_t)H.N * c + 255) & ~size_t(255)) / 8;
  P.scratch.alloc(8 * 5 * stride, st);
  double* scratch = P.scratch.as<double>();
  // pinned host X / Y are read and written by the first and last steps
  // directly (measured faster than copy nodes staging them in the graph)
  const std::vector<StepRec<double>> steps =
      trans ? solve_steps_T<double>(H, X, ldx, Y, ldy, c, scratch, stride)
            : solve_steps<double>(H, X, ldx, Y, ldy, c, scratch, stride);
  const std::vector<PlanKnobs>* kn = nullptr;
  if (!trans) {
    auto it = H.tuned.find({type_code<double>(), c});
    if (it != H.tuned.end() && it->second.size() == steps.size()) kn = &it->second;
  }
  for (size_t i = 0; i < steps.size(); ++i)
    sweep::prepare_step(steps[i].s, kn ? (*kn)[i] : PlanKnobs());
  stream_wait(st);   // the scratch exists before the capture
  // capture on a private stream (the caller's may be the legacy default
  // stream, which cannot be captured); the graph launches on the caller's
  cudaStream_t cs = nullptr;
  SLU_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  const long long n0 = launch_thread();
  try {
    SLU_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
      for (size_t i = 0; i < steps.size(); ++i)
        launch_step(cs, steps[i].s, steps[i].what, nullptr, 0, 0, kn ? (*kn)[i] : PlanKnobs());
    } catch (...) {
      cudaStreamEndCapture(cs, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    SLU_CHECK_CUDA(cudaStreamEndCapture(cs, &g));
    // captured launches run when the graph is replayed: count them there
    P.kernels = launch_thread() - n0;
    launch_total() -= P.kernels;
    launch_thread() = n0;
    const cudaError_t e = cudaGraphInstantiate(&P.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
      throw Error(SLU_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  } catch (...) {
    cudaStreamDestroy(cs);
    throw;
  }
  SLU_CHECK_CUDA(cudaStreamDestroy(cs));
  P.H = {&H};
  P.alive = {H.alive};
  P.gen = {H.sweep_gen};
}

void solve_plan_launch(Handle& h, SolvePlan& P, bool wait) {
  for (size_t i = 0; i < P.H.size(); ++i) {
    if (P.alive[i].expired())
      throw Error(SLU_ERR_STATE, "an operator of the solve plan was destroyed");
    if (P.H[i]->sweep_gen != P.gen[i])
      throw Error(SLU_ERR_STATE, "an operator was refactored after the solve plan was made");
  }
  if (!P.exec) return;   // a grouped plan without members
  SLU_CHECK_CUDA(cudaGraphLaunch(P.exec, h.stream));
  count_launches(P.kernels);
  if (wait) stream_wait(h.stream);
}

namespace {

// Coordinate descent on the whole solve: starting from the default caps,
// each launch in turn tries every candidate cap set that changes its plan;
// a candidate is kept when the median time of `reps` full solves (CUDA events
// around the solve, programmatic dependent launch as in use) drops by more
// than 0.5%.  Timing whole solves keeps the overlap between consecutive
// launches in the measurement.  The buffers hold zeros: every launch reads
// and writes finite values, and timing does not depend on the data.
template <typename T>
void autotune(Handle& h, Hbs& H, int c, int reps) {
  cudaStream_t st = h.stream;
  const size_t n = (size_t)H.N * c;
  const size_t stride = ((sizeof(T) * n + 255) & ~size_t(255)) / sizeof(T);
  DevBuf buf;
  buf.alloc(sizeof(T) * 6 * stride, st);
  SLU_CHECK_CUDA(cudaMemsetAsync(buf.p, 0, sizeof(T) * 6 * stride, st));
  T* B = buf.as<T>();
  const std::vector<StepRec<T>> steps = solve_steps<T>(H, B, c, B, c, c, B + stride, stride);
  std::vector<PlanKnobs> cand;
  for (int target : {1, 2, 4})
    for (int rmin : {8, 16, 32, 64})
      for (int cmax : {8, 16, 32, 64}) cand.push_back({target, rmin, cmax});
  cudaEvent_t e0, e1;
  SLU_CHECK_CUDA(cudaEventCreate(&e0));
  SLU_CHECK_CUDA(cudaEventCreate(&e1));
  std::vector<PlanKnobs> cur(steps.size());
  auto measure = [&](const std::vector<PlanKnobs>& kn) {
    std::vector<float> ms;
    for (int r = 0; r < reps; ++r) {
      SLU_CHECK_CUDA(cudaEventRecord(e0, st));
      for (size_t i = 0; i < steps.size(); ++i)
        launch_step(st, steps[i].s, steps[i].what, nullptr, 0, 0, kn[i]);
      SLU_CHECK_CUDA(cudaEventRecord(e1, st));
      SLU_CHECK_CUDA(cudaEventSynchronize(e1));
      float x = 0.f;
      SLU_CHECK_CUDA(cudaEventElapsedTime(&x, e0, e1));
      ms.push_back(x);
    }
    std::nth_element(ms.begin(), ms.begin() + ms.size() / 2, ms.end());
    return ms[ms.size() / 2];
  };
  try {
    measure(cur);   // warm-up (kernel attributes, caches)
    float best = measure(cur);
    for (size_t i = 0; i < steps.size(); ++i) {
      std::vector<std::array<long long, 4>> seen;
      {
        sweep::Step<T> t = steps[i].s;
        sweep::Step<T>* one = &t;
        const sweep::LaunchPlan p = sweep::plan_steps(&one, 1, cur[i]);
        seen.push_back({t.rch, t.cpb, p.threads, p.ctas});
      }
      for (const PlanKnobs& k : cand) {
        sweep::Step<T> t = steps[i].s;
        sweep::Step<T>* one = &t;
        const sweep::LaunchPlan p = sweep::plan_steps(&one, 1, k);
        const std::array<long long, 4> key{t.rch, t.cpb, p.threads, p.ctas};
        if (std::find(seen.begin(), seen.end(), key) != seen.end()) continue;
        seen.push_back(key);
        std::vector<PlanKnobs> trial = cur;
        trial[i] = k;
        const float ms = measure(trial);
        if (ms < 0.995f * best) {
          best = ms;
          cur = trial;
        }
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  stream_wait(st);
  H.tuned[{type_code<T>(), c}] = cur;
}

}  // namespace

void hbs_autotune_solve(Handle& h, Hbs& H, int c, int precision, int reps) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  SLU_REQUIRE(c >= 1 && reps >= 1, "bad arguments");
  if (precision == 0) {
    autotune<double>(h, H, c, reps);
  } else if (precision == 2) {
    if (!H.has_dfs) hbs_make_dfs(h, H);
    autotune<dfloat>(h, H, c, reps);
  } else {
    throw Error(SLU_ERR_ARG, "autotune precision must be 0 (float64) or 2 (double-float)");
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
                                      LaunchTimes*, const double*, int);
template void ulv_solve_fused<float>(cudaStream_t, const Hbs&, float*, int, int, float*, size_t,
                                     LaunchTimes*, const float*, int);
template void ulv_solve_fused<dfloat>(cudaStream_t, const Hbs&, dfloat*, int, int, dfloat*, size_t,
                                      LaunchTimes*, const dfloat*, int);

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
  if (H.top >= 1) split_dfs(st, H.Top, H.Topdf);
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
