// Mixed-precision refinement of the HBS solve, replayed as CUDA graphs.
//
//   x0 = inner ULV solve of b;  r = b - A x  (double-float apply)
//   x += inner ULV solve of r;  r = b - A x  ...
// until ||r_j|| / ||b_j|| <= tol for every column j.  The inner sweep runs on
// the float32 pipe: either in double-float arithmetic (the default; ~1e-14
// relative, so one iteration usually reaches the tolerance) or in plain
// float32 (two or three iterations).
//
// One refinement iteration (cast, inner fused ULV sweep, correction, double-
// float residual, column norms, device-to-host copy of the norms) is captured
// once per (operator, nrhs) into a CUDA graph over buffers that the plan owns,
// and replayed.  With the float32 inner sweep the host looks at the norms only
// from the second correction on (a float32 solve alone never reaches a
// float64 tolerance).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "abi_types.cuh"
#include "refine_kernels.cuh"

namespace slu {

struct RefinePlan {
  int c = 0;
  int inner = 0;   // 0 float32 sweep (f), 1 double-float sweep (d), 2 tensor-core sweep
  DevBuf B, X, r, f, d, bn, rn, solve_ws, df_ws, ozerr;
  double* host_norms = nullptr;   // pinned: [bn (c) | rn (c) | error word]
  cudaGraphExec_t first = nullptr, next = nullptr;
  long long first_kernels = 0, next_kernels = 0;   // kernel nodes per graph
  ~RefinePlan() {
    if (first) cudaGraphExecDestroy(first);
    if (next) cudaGraphExecDestroy(next);
    if (host_norms) cudaFreeHost(host_norms);
  }
};

namespace {

// One refinement iteration.  Bc / Xc (leading dimension c) replace the plan's
// B and X buffers when given (the tensor-core inner mode's direct path).
void enqueue_iteration(cudaStream_t st, const Hbs& H, RefinePlan& P, bool first,
                       const double* Bc = nullptr, double* Xc = nullptr) {
  const int N = H.N, c = P.c;
  const long long n = (long long)N * c;
  const double* B = Bc ? Bc : P.B.as<double>();
  double* X = Xc ? Xc : P.X.as<double>();
  double* r = P.r.as<double>();
  if (first) {
    if (P.inner == 2) {
      SLU_CHECK_CUDA(cudaMemsetAsync(P.bn.p, 0, 8 * (size_t)c, st));
      colsumsq_k<<<dim3((c + 127) / 128, std::min(64, std::max(1, N / 64))), 128, 0, st>>>(
          N, c, B, c, P.bn.as<double>());
      check_launch("colsumsq_k");
    } else {
      colnorm2_k<<<c, 256, 0, st>>>(N, c, B, c, P.bn.as<double>());
      check_launch("colnorm2_k");
    }
    SLU_CHECK_CUDA(cudaMemcpyAsync(P.host_norms, P.bn.p, 8 * c, cudaMemcpyDeviceToHost, st));
  }
  const double* rhs = first ? B : r;
  if (P.inner == 2) {
    // tensor-core sweep and residual (ozaki.cu): the first solve writes X in
    // float64 directly; corrections come back as double-float pairs
    unsigned* err = P.ozerr.as<unsigned>();
    double* d = P.d.as<double>();
    if (first) {
      ulv_solve_oz(st, H, rhs, c, X, c, c, P.solve_ws.p, err);
    } else {
      ulv_solve_oz(st, H, rhs, c, d, c, c, P.solve_ws.p, err);
      add_k<<<gsz(n), 256, 0, st>>>(n, d, X);
      check_launch("add_k");
    }
    // r = B - A X straight from the apply's last step, with its column norms
    SLU_CHECK_CUDA(cudaMemsetAsync(P.rn.p, 0, 8 * (size_t)c, st));
    hbs_apply_oz(st, H, X, c, r, c, c, P.solve_ws.p, err, B, P.rn.as<double>());
    SLU_CHECK_CUDA(cudaMemcpyAsync(P.host_norms + c, P.rn.p, 8 * c, cudaMemcpyDeviceToHost, st));
    SLU_CHECK_CUDA(cudaMemcpyAsync(P.host_norms + 2 * c, P.ozerr.p, 8, cudaMemcpyDeviceToHost,
                                   st));
    return;
  }
  if (P.inner == 1) {
    dfloat* d = P.d.as<dfloat>();
    to_dfs_k<<<gsz(n), 256, 0, st>>>(n, rhs, d);
    check_launch("to_dfs_k");
    const size_t stride =
        ((sizeof(dfloat) * (size_t)N * c + 255) & ~size_t(255)) / sizeof(dfloat);
    ulv_solve_fused<dfloat>(st, H, d, c, c, P.solve_ws.as<dfloat>(), stride);
    accum_dfs_k<<<gsz(n), 256, 0, st>>>(n, d, X, first ? 1 : 0);
    check_launch("accum_dfs_k");
  } else {
    float* f = P.f.as<float>();
    to_f32_k<<<gsz(n), 256, 0, st>>>(n, rhs, f);
    check_launch("to_f32_k");
    hbs_solve_scratch<float>(st, H, false, f, c, c, P.solve_ws.as<float>());
    accum_k<<<gsz(n), 256, 0, st>>>(n, f, X, first ? 1 : 0);
    check_launch("accum_k");
  }
  hbs_apply_df(st, H, X, c, r, c, c, P.df_ws.p);
  resid_k<<<gsz(n), 256, 0, st>>>(n, B, r);
  check_launch("resid_k");
  colnorm2_k<<<c, 256, 0, st>>>(N, c, r, c, P.rn.as<double>());
  check_launch("colnorm2_k");
  SLU_CHECK_CUDA(cudaMemcpyAsync(P.host_norms + c, P.rn.p, 8 * c, cudaMemcpyDeviceToHost, st));
}

cudaGraphExec_t capture(cudaStream_t st, const Hbs& H, RefinePlan& P, bool first) {
  cudaGraph_t g = nullptr;
  SLU_CHECK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const long long n0 = launch_thread();
  try {
    enqueue_iteration(st, H, P, first);
    // captured launches run when the graph is replayed: count them there
    const long long d = launch_thread() - n0;
    (first ? P.first_kernels : P.next_kernels) = d;
    launch_thread() = n0;
    launch_total() -= d;
  } catch (...) {
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  SLU_CHECK_CUDA(cudaStreamEndCapture(st, &g));
  cudaGraphExec_t ex = nullptr;
  cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    throw Error(SLU_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return ex;
}

RefinePlan& plan_for(Handle& h, Hbs& H, int c) {
  auto it = H.refine_plans.find(c);
  if (it != H.refine_plans.end()) return *it->second;
  cudaStream_t st = h.stream;
  auto P = std::make_shared<RefinePlan>();
  P->c = c;
  P->inner = H.refine_inner;
  const size_t n = (size_t)H.N * c;
  P->B.alloc(8 * n, st);
  P->X.alloc(8 * n, st);
  P->r.alloc(8 * n, st);
  if (P->inner >= 1) P->d.alloc(8 * n, st);
  else P->f.alloc(4 * n, st);
  P->bn.alloc(8 * (size_t)c, st);
  P->rn.alloc(8 * (size_t)c, st);
  if (P->inner == 2) {
    P->solve_ws.alloc(hbs_oz_scratch_bytes(H, c), st);
    P->ozerr.alloc(8, st);
    SLU_CHECK_CUDA(cudaMemsetAsync(P->ozerr.p, 0, 8, st));
  } else {
    P->solve_ws.alloc(hbs_solve_scratch_bytes(H, c, P->inner == 1 ? 8 : 4), st);
    P->df_ws.alloc(hbs_apply_df_scratch_bytes(H, c), st);
  }
  SLU_CHECK_CUDA(cudaMallocHost(&P->host_norms, 16 * (size_t)c + 16));
  P->host_norms[2 * c] = 0.0;
  stream_wait(st);
  // an uncaptured run first: sets kernel attributes and validates the sequence
  SLU_CHECK_CUDA(cudaMemsetAsync(P->B.p, 0, 8 * n, st));
  enqueue_iteration(st, H, *P, true);
  stream_wait(st);
  // capture on a private stream (the caller's may be the legacy default
  // stream, which cannot be captured); the graphs launch on the caller's
  cudaStream_t cs = nullptr;
  SLU_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  try {
    P->first = capture(cs, H, *P, true);
    P->next = capture(cs, H, *P, false);
  } catch (...) {
    cudaStreamDestroy(cs);
    throw;
  }
  SLU_CHECK_CUDA(cudaStreamDestroy(cs));
  RefinePlan& ref = *P;
  H.refine_plans[c] = P;
  return ref;
}

}  // namespace

void hbs_refine(Handle& h, Hbs& H, const double* B, int ldb, double* X, int ldx, int c,
                double tol, int maxit, int* iters, double* relres) {
  cudaStream_t st = h.stream;
  if (H.refine_inner == 2) {
    if (!H.has_oz) hbs_make_oz(h, H);
  } else {
    if (H.refine_inner == 1 && !H.has_dfs) hbs_make_dfs(h, H);
    if (H.refine_inner == 0 && !H.has_f32) hbs_make_f32(h, H);
    if (!H.has_df) hbs_make_df(h, H);
  }
  RefinePlan& P = plan_for(h, H, c);
  // the tensor-core mode on dense caller blocks runs its iterations straight
  // on the caller's B and X: its launches are long enough that the graph's
  // launch savings do not pay for staging copies of B and X
  const bool direct = P.inner == 2 && ldb == c && ldx == c;
  if (direct) {
    enqueue_iteration(st, H, P, true, B, X);
  } else {
    SLU_CHECK_CUDA(cudaMemcpy2DAsync(P.B.p, 8 * (size_t)c, B, 8 * (size_t)ldb, 8 * (size_t)c,
                                     H.N, cudaMemcpyDeviceToDevice, st));
    SLU_CHECK_CUDA(cudaGraphLaunch(P.first, st));
    count_launches(P.first_kernels);
  }
  int it = 1;
  double worst = 0.0;
  for (;;) {
    if (P.inner == 0 && it < 2 && it < maxit && tol < 1e-6) {  // float32: no check yet
      SLU_CHECK_CUDA(cudaGraphLaunch(P.next, st));
      count_launches(P.next_kernels);
      ++it;
      continue;
    }
    stream_wait(st);
    if (P.inner == 2) {
      unsigned long long ew = 0;
      std::memcpy(&ew, P.host_norms + 2 * c, 8);
      if (ew != 0) {
        SLU_CHECK_CUDA(cudaMemsetAsync(P.ozerr.p, 0, 8, st));
        P.host_norms[2 * c] = 0.0;
        throw Error(SLU_ERR_TIMEOUT, "tensor-core sweep: a device wait timed out");
      }
    }
    worst = 0.0;
    for (int j = 0; j < c; ++j) {
      const double bj = P.host_norms[j], rj = P.host_norms[c + j];
      worst = std::max(worst, std::sqrt(rj) / (bj > 0 ? std::sqrt(bj) : 1.0));
    }
    if (worst <= tol || it >= maxit) break;
    if (direct) {
      enqueue_iteration(st, H, P, false, B, X);
    } else {
      SLU_CHECK_CUDA(cudaGraphLaunch(P.next, st));
      count_launches(P.next_kernels);
    }
    ++it;
  }
  if (!direct)
    SLU_CHECK_CUDA(cudaMemcpy2DAsync(X, 8 * (size_t)ldx, P.X.p, 8 * (size_t)c, 8 * (size_t)c,
                                     H.N, cudaMemcpyDeviceToDevice, st));
  if (iters) *iters = it;
  if (relres) *relres = worst;
  if (worst > tol) throw Error(SLU_ERR_NOT_CONVERGED, "refinement did not reach the tolerance");
}

}  // namespace slu
