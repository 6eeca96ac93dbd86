// extern "C" boundary of libslablu (declared in include/slablu.h).
// Every entry point catches slu::Error / std::exception and returns a status
// code; the message is kept per thread for slu_last_error().
#include <cstring>
#include <memory>
#include <string>

#include "abi_types.cuh"

namespace slu {
std::string& thread_error() {
  static thread_local std::string msg;
  return msg;
}
}  // namespace slu

namespace {
#define g_err (slu::thread_error())

template <class F>
int guard(slu_handle_t h, F&& f) {
  return slu::guard_call(h, static_cast<F&&>(f));
}

}  // namespace

extern "C" {

int slu_version(void) { return 1; }

long long slu_launch_count(void) { return slu::launch_total().load(); }

void slu_set_blocking_waits(int on) { slu::set_blocking_waits(on != 0); }

int slu_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return SLU_ERR_ARG;
  std::strncpy(buf, g_err.c_str(), len - 1);
  buf[len - 1] = '\0';
  return SLU_OK;
}

int slu_create(void* stream, slu_handle_t* out) {
  return guard(nullptr, [&] {
    SLU_REQUIRE(out, "null output pointer");
    auto p = std::make_unique<slu_handle_s>();
    p->h.stream = reinterpret_cast<cudaStream_t>(stream);
    p->h.info.alloc(64 * sizeof(int), p->h.stream);
    SLU_CHECK_CUDA(cudaMemsetAsync(p->h.info.p, 0, 64 * sizeof(int), p->h.stream));
    *out = p.release();
  });
}

int slu_destroy(slu_handle_t h) {
  return guard(nullptr, [&] {
    if (!h) return;
    cudaStreamSynchronize(h->h.stream);
    delete h;
  });
}

int slu_set_stream(slu_handle_t h, void* stream) {
  return guard(h, [&] {
    SLU_REQUIRE(h, "null handle");
    slu::stream_wait(h->h.stream);
    h->h.stream = reinterpret_cast<cudaStream_t>(stream);
  });
}

int slu_sync(slu_handle_t h) {
  int st = guard(h, [&] {
    SLU_REQUIRE(h, "null handle");
    slu::stream_wait(h->h.stream);
  });
  if (st != SLU_OK) return st;
  int info[64];
  st = guard(h, [&] {
    SLU_CHECK_CUDA(cudaMemcpy(info, h->h.info.p, sizeof(info), cudaMemcpyDeviceToHost));
  });
  if (st != SLU_OK) return st;
  if (info[1] != 0) {
    cudaMemset(h->h.info.p, 0, sizeof(info));
    g_err = "a tensor-core GEMM gave up waiting on its TMA / MMA pipeline";
    h->h.last_error = g_err;
    return SLU_ERR_TIMEOUT;
  }
  if (info[0] != 0) {
    cudaMemset(h->h.info.p, 0, sizeof(info));
    g_err = "a device-side factorisation reported a failure (zero pivot or Jacobi sweep limit)";
    h->h.last_error = g_err;
    return SLU_ERR_NOT_CONVERGED;
  }
  return SLU_OK;
}

// ------------------------------------------------------------------ HBS
int slu_hbs_create(slu_handle_t h, int N, int L, int fac, const int64_t* perm_host,
                   slu_hbs_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && out, "null argument");
    SLU_REQUIRE(N > 0 && L >= 1 && (fac == 2 || fac == 4), "bad HBS geometry");
    auto p = std::make_unique<slu_hbs_s>();
    p->H.N = N;
    p->H.L = L;
    p->H.fac = fac;
    std::vector<int64_t> perm(N);
    bool ident = true;
    if (perm_host) {
      std::vector<char> seen(N, 0);
      for (int i = 0; i < N; ++i) {
        int64_t v = perm_host[i];
        SLU_REQUIRE(v >= 0 && v < N && !seen[v], "perm is not a permutation of 0..N-1");
        seen[v] = 1;
        perm[i] = v;
        ident = ident && (v == i);
      }
    } else {
      for (int i = 0; i < N; ++i) perm[i] = i;
    }
    p->H.identity_perm = ident;
    p->H.perm.alloc(sizeof(int64_t) * N, h->h.stream);
    SLU_CHECK_CUDA(cudaMemcpyAsync(p->H.perm.p, perm.data(), sizeof(int64_t) * N,
                                   cudaMemcpyHostToDevice, h->h.stream));
    // the mode-T solve scatters its input and gathers its output through perm
    // (HBSnew.py:403-411): as step gathers / scatters that is the inverse
    std::vector<int64_t> iperm(N);
    for (int i = 0; i < N; ++i) iperm[perm[i]] = i;
    p->H.iperm.alloc(sizeof(int64_t) * N, h->h.stream);
    SLU_CHECK_CUDA(cudaMemcpyAsync(p->H.iperm.p, iperm.data(), sizeof(int64_t) * N,
                                   cudaMemcpyHostToDevice, h->h.stream));
    slu::stream_wait(h->h.stream);
    p->H.lv.resize(L);
    *out = p.release();
  });
}

int slu_hbs_destroy(slu_hbs_t op) {
  return guard(nullptr, [&] { delete op; });
}

int slu_hbs_compress(slu_handle_t h, slu_hbs_t op, int nleaves, int rk, int s, const double* Om,
                     const double* Psi, const double* Y, const double* Z, int compute_ulv) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && Om && Psi && Y && Z, "null argument");
    SLU_REQUIRE(s >= 1, "bad sample count");
    slu::hbs_compress(h->h, op->H, nleaves, rk, s, Om, Psi, Y, Z, compute_ulv != 0);
  });
}

int slu_hbs_set_level(slu_handle_t h, slu_hbs_t op, int level, int Nb, int n, int k,
                      const double* U, const double* V, const double* D) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && D, "null argument");
    slu::Hbs& H = op->H;
    SLU_REQUIRE(level >= 0 && level < H.L, "level out of range");
    const bool root = (level == H.L - 1);
    SLU_REQUIRE(Nb >= 1 && n >= 1 && k >= 0 && k <= n, "bad level geometry");
    SLU_REQUIRE(root ? (k == 0 && Nb == 1) : (k >= 1 && U), "root takes k = 0, others U (and V)");
    if (level == 0) SLU_REQUIRE((long long)Nb * n == H.N, "leaf level must cover N rows");
    cudaStream_t st = h->h.stream;
    slu::Level& l = H.lv[level];
    l = slu::Level();
    l.Nb = Nb;
    l.n = n;
    l.k = k;
    const size_t rows = (size_t)Nb * n;
    if (!root) {
      l.U.alloc(8 * rows * k, st);
      SLU_CHECK_CUDA(cudaMemcpyAsync(l.U.p, U, 8 * rows * k, cudaMemcpyDeviceToDevice, st));
      if (V) {  // V is needed for apply and factorisation, not for a solve of loaded factors
        l.V.alloc(8 * rows * k, st);
        SLU_CHECK_CUDA(cudaMemcpyAsync(l.V.p, V, 8 * rows * k, cudaMemcpyDeviceToDevice, st));
      }
    }
    l.D.alloc(8 * rows * n, st);
    SLU_CHECK_CUDA(cudaMemcpyAsync(l.D.p, D, 8 * rows * n, cudaMemcpyDeviceToDevice, st));
    // geometry is complete once every level is set
    bool all = true;
    for (const slu::Level& x : H.lv) all = all && x.D.p;
    if (all) {
      for (int t = 1; t < H.L; ++t) {
        SLU_REQUIRE(H.lv[t].n == H.fac * H.lv[t - 1].k &&
                        H.lv[t].Nb * H.fac == H.lv[t - 1].Nb,
                    "inconsistent HBS level shapes");
      }
      H.NN.assign(H.L + 1, 0);
      for (int t = 0; t < H.L; ++t) {
        slu::Level& x = H.lv[t];
        x.nu = (t == H.L - 1) ? x.n : x.n - x.k;
        H.NN[t + 1] = H.NN[t] + (long long)x.nu * x.Nb;
      }
      H.has_mats = true;
      H.has_ulv = false;
      H.has_sweep = false;
      H.has_oz = H.has_ozT = false;
      H.has_f32 = false;
      H.has_dfs = false;
      H.has_df = false;
      H.has_apply[0] = H.has_apply[1] = false;
      H.invalidate_plans();
    }
  });
}

int slu_hbs_set_ulv_level(slu_handle_t h, slu_hbs_t op, int level, const double* Q,
                          const double* W, const double* R, const double* Uu) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_mats, "set every level with slu_hbs_set_level first");
    SLU_REQUIRE(level >= 0 && level < H.L, "level out of range");
    const bool root = (level == H.L - 1);
    cudaStream_t st = h->h.stream;
    slu::Level& l = H.lv[level];
    const size_t rows = (size_t)l.Nb * l.n;
    l.kU = root ? 0 : l.k;
    l.uu_rows = root ? 0 : l.n - l.k;
    // a factor with no entries (n = k: no eliminated rows, empty R and Uu)
    // may come as a null pointer
    SLU_REQUIRE(Q || rows * l.n == 0, "null Q");
    SLU_REQUIRE(R || (size_t)l.Nb * l.nu * l.n == 0, "null R");
    SLU_REQUIRE(root || W || rows * l.n == 0, "non-root levels need W");
    SLU_REQUIRE(root || Uu || (size_t)l.Nb * l.uu_rows * l.kU == 0, "non-root levels need Uu");
    auto put = [&](slu::DevBuf& b, const double* src, size_t count) {
      b.alloc(8 * count, st);
      if (count) SLU_CHECK_CUDA(cudaMemcpyAsync(b.p, src, 8 * count, cudaMemcpyDeviceToDevice, st));
    };
    put(l.Q, Q, rows * l.n);
    put(l.R, R, (size_t)l.Nb * l.nu * l.n);
    if (!root) {
      put(l.W, W, rows * l.n);
      put(l.Uu, Uu, (size_t)l.Nb * l.uu_rows * l.kU);
    }
    l.Uf.release(); l.Df.release(); l.Qf.release(); l.Wf.release(); l.Rf.release(); l.Uuf.release();
    bool all = true;
    for (int t = 0; t < H.L; ++t)
      all = all && H.lv[t].Q.p && (H.lv[t].R.p || (size_t)H.lv[t].Nb * H.lv[t].nu == 0);
    H.has_ulv = all;
    H.has_f32 = false;
    H.has_dfs = false;
    H.has_sweep = false;
    H.has_oz = H.has_ozT = false;
    H.invalidate_plans();
    if (all) slu::hbs_make_sweep(h->h, H);
  });
}

int slu_ulv_factor(slu_handle_t h, slu_hbs_t op) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    slu::hbs_factor(h->h, op->H);
  });
}

int slu_hbs_apply(slu_handle_t h, slu_hbs_t op, int trans, const double* X, int ldx, double* Y,
                  int ldy, int nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && X && Y, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldx >= nrhs && ldy >= nrhs, "bad right-hand side shape");
    slu::hbs_apply(h->h, op->H, trans != 0, X, ldx, Y, ldy, nrhs);
  });
}

int slu_ulv_solve(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs, int trans) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && B, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    slu::hbs_solve<double>(h->h, op->H, trans != 0, B, ldb, nrhs);
  });
}

int slu_ulv_solve_into(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                       int ldy, int nrhs, int trans) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && X && Y, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldx >= nrhs && ldy >= nrhs, "bad right-hand side shape");
    const slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    cudaStream_t st = h->h.stream;
    const size_t bytes = slu::hbs_solve_scratch_bytes(H, nrhs, sizeof(double));
    h->h.ws.reserve(bytes + 256, st);
    double* scratch = h->h.ws.take<double>(bytes / sizeof(double));
    const size_t stride = ((sizeof(double) * (size_t)H.N * nrhs + 255) & ~size_t(255)) / 8;
    if (trans) slu::ulv_solve_T<double>(st, H, Y, ldy, nrhs, scratch, stride, X, ldx);
    else slu::ulv_solve_fused<double>(st, H, Y, ldy, nrhs, scratch, stride, nullptr, X, ldx);
  });
}

int slu_ulv_solve_plan_create(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                              int ldy, int nrhs, int trans, slu_solve_plan_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && X && Y && out, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldx >= nrhs && ldy >= nrhs, "bad right-hand side shape");
    SLU_REQUIRE(op->H.has_ulv, "HBS operator has no ULV factorisation");
    auto p = std::make_unique<slu_solve_plan_s>();
    slu::solve_plan_create(h->h, op->H, X, ldx, Y, ldy, nrhs, trans != 0, p->P);
    *out = p.release();
  });
}

int slu_ulv_solve_grouped_plan_create(slu_handle_t h, int count, const slu_hbs_t* ops,
                                      double* const* B, const int* ldb, const int* nrhs,
                                      slu_solve_plan_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && out, "null argument");
    SLU_REQUIRE(count >= 0 && (count == 0 || ops), "null argument");
    std::vector<slu::Hbs*> H(count);
    for (int i = 0; i < count; ++i) {
      SLU_REQUIRE(ops[i], "null operator");
      H[i] = &ops[i]->H;
    }
    auto p = std::make_unique<slu_solve_plan_s>();
    slu::grouped_solve_plan_create(h->h, count, H.data(), B, ldb, nrhs, p->P);
    *out = p.release();
  });
}

int slu_grouped_program_create(slu_handle_t h, int nphase, const int* kind, const int* count,
                               const slu_hbs_t* ops, double* const* X, double* const* Y,
                               const int* ld, const int* nrhs, const long long* n,
                               slu_solve_plan_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && out, "null argument");
    SLU_REQUIRE(nphase >= 0 && (nphase == 0 || (kind && count)), "null argument");
    long long total = 0;
    for (int p = 0; p < nphase; ++p) total += count[p];
    std::vector<slu::Hbs*> H(total, nullptr);
    if (ops)
      for (long long i = 0; i < total; ++i) H[i] = ops[i] ? &ops[i]->H : nullptr;
    auto p = std::make_unique<slu_solve_plan_s>();
    slu::grouped_program_create(h->h, nphase, kind, count, ops ? H.data() : nullptr, X, Y, ld,
                                nrhs, n, p->P);
    *out = p.release();
  });
}

int slu_ulv_solve_plan_launch(slu_handle_t h, slu_solve_plan_t plan, int wait) {
  return guard(h, [&] {
    SLU_REQUIRE(h && plan, "null argument");
    slu::solve_plan_launch(h->h, plan->P, wait != 0);
  });
}

int slu_ulv_solve_plan_destroy(slu_solve_plan_t plan) {
  return guard(nullptr, [&] { delete plan; });
}

int slu_hbs_prepare_f32(slu_handle_t h, slu_hbs_t op) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    slu::hbs_make_f32(h->h, op->H);
  });
}

int slu_ulv_solve_f32(slu_handle_t h, slu_hbs_t op, float* B, int ldb, int nrhs, int trans) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && B, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    slu::hbs_solve<float>(h->h, op->H, trans != 0, B, ldb, nrhs);
  });
}

int slu_hbs_prepare_dfloat(slu_handle_t h, slu_hbs_t op) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    slu::hbs_make_dfs(h->h, op->H);
  });
}

int slu_ulv_solve_dfloat(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && B, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    if (!H.has_dfs) slu::hbs_make_dfs(h->h, H);
    const size_t bytes = slu::hbs_solve_df_scratch_bytes(H, nrhs);
    h->h.ws.reserve(bytes + 256, h->h.stream);
    void* scratch = h->h.ws.take<char>(bytes);
    slu::hbs_solve_df(h->h.stream, H, B, ldb, nrhs, scratch);
  });
}

int slu_hbs_prepare_ozaki(slu_handle_t h, slu_hbs_t op) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    SLU_REQUIRE(op->H.has_ulv, "HBS operator has no ULV factorisation");
    slu::hbs_make_oz(h->h, op->H);
  });
}

int slu_ulv_solve_ozaki(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                        int ldy, int nrhs, int trans) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && X && Y, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldx >= nrhs && ldy >= nrhs, "bad right-hand side shape");
    slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    if (trans ? !H.has_ozT : !H.has_oz) (trans ? slu::hbs_make_ozT : slu::hbs_make_oz)(h->h, H);
    const size_t bytes = slu::hbs_oz_scratch_bytes(H, nrhs);
    h->h.ws.reserve(bytes + 256, h->h.stream);
    void* scratch = h->h.ws.take<char>(bytes);
    unsigned* err = reinterpret_cast<unsigned int*>(h->h.info.as<int>()) + 1;
    if (trans)
      slu::ulv_solve_oz_T(h->h.stream, H, X, ldx, Y, ldy, nrhs, scratch, err);
    else
      slu::ulv_solve_oz(h->h.stream, H, X, ldx, Y, ldy, nrhs, scratch, err);
  });
}

int slu_hbs_apply_ozaki(slu_handle_t h, slu_hbs_t op, const double* X, int ldx, double* Y,
                        int ldy, int nrhs, int trans) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && X && Y, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldx >= nrhs && ldy >= nrhs, "bad right-hand side shape");
    slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    if (trans ? !H.has_ozT : !H.has_oz) (trans ? slu::hbs_make_ozT : slu::hbs_make_oz)(h->h, H);
    const size_t bytes = slu::hbs_oz_scratch_bytes(H, nrhs);
    h->h.ws.reserve(bytes + 256, h->h.stream);
    void* scratch = h->h.ws.take<char>(bytes);
    slu::hbs_apply_oz(h->h.stream, H, X, ldx, Y, ldy, nrhs, scratch,
                      reinterpret_cast<unsigned int*>(h->h.info.as<int>()) + 1, nullptr, nullptr,
                      trans != 0);
  });
}

int slu_hbs_set_refine_inner(slu_hbs_t op, int mode) {
  return guard(nullptr, [&] {
    SLU_REQUIRE(op, "null argument");
    SLU_REQUIRE(mode >= 0 && mode <= 2, "refine inner mode must be 0, 1 or 2");
    if (op->H.refine_inner != mode) op->H.invalidate_plans();
    op->H.refine_inner = mode;
  });
}

int slu_refine(slu_handle_t h, slu_hbs_t op, const double* B, int ldb, double* X, int ldx,
               int nrhs, double tol, int maxit, int* iters_out, double* relres_out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && B && X, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs && ldx >= nrhs && maxit >= 1, "bad arguments");
    slu::hbs_refine(h->h, op->H, B, ldb, X, ldx, nrhs, tol, maxit, iters_out, relres_out);
  });
}

namespace {
std::vector<slu::Hbs*> group_ops(int count, const slu_hbs_t* ops) {
  SLU_REQUIRE(count >= 0 && (count == 0 || ops), "null argument");
  std::vector<slu::Hbs*> H(count);
  for (int i = 0; i < count; ++i) {
    SLU_REQUIRE(ops[i], "null operator");
    H[i] = &ops[i]->H;
  }
  return H;
}
}  // namespace

int slu_refine_grouped_plan_create(slu_handle_t h, int count, const slu_hbs_t* ops,
                                   const double* const* B, const int* ldb, double* const* X,
                                   const int* ldx, const int* nrhs, slu_refine_plan_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && out, "null argument");
    std::vector<slu::Hbs*> H = group_ops(count, ops);
    auto p = std::make_unique<slu_refine_plan_s>();
    p->P = slu::grouped_refine_plan_create(h->h, count, H.data(), B, ldb, X, ldx, nrhs);
    *out = p.release();
  });
}

int slu_refine_plan_run(slu_handle_t h, slu_refine_plan_t plan, double tol, int maxit,
                        int* iters_out, double* relres_out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && plan && plan->P, "null argument");
    plan->P->run(h->h, tol, maxit, iters_out, relres_out);
  });
}

int slu_refine_plan_destroy(slu_refine_plan_t plan) {
  return guard(nullptr, [&] { delete plan; });
}

int slu_ulv_solve_grouped(slu_handle_t h, int count, const slu_hbs_t* ops, double* const* B,
                          const int* ldb, const int* nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h, "null argument");
    std::vector<slu::Hbs*> H = group_ops(count, ops);
    slu::hbs_solve_grouped(h->h, count, H.data(), B, ldb, nrhs);
  });
}

int slu_hbs_apply_grouped(slu_handle_t h, int count, const slu_hbs_t* ops, const int* trans,
                          const double* const* X, const int* ldx, double* const* Y,
                          const int* ldy, const int* nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h, "null argument");
    std::vector<slu::Hbs*> H = group_ops(count, ops);
    slu::hbs_apply_grouped(h->h, count, H.data(), trans, X, ldx, Y, ldy, nrhs);
  });
}

int slu_refine_grouped(slu_handle_t h, int count, const slu_hbs_t* ops, const double* const* B,
                       const int* ldb, double* const* X, const int* ldx, const int* nrhs,
                       double tol, int maxit, int* iters_out, double* relres_out) {
  return guard(h, [&] {
    SLU_REQUIRE(h, "null argument");
    std::vector<slu::Hbs*> H = group_ops(count, ops);
    slu::hbs_refine_grouped(h->h, count, H.data(), B, ldb, X, ldx, nrhs, tol, maxit, iters_out,
                            relres_out);
  });
}

int slu_ulv_solve_timed(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs,
                        float* ms_out, int* level_out, int* kind_out, int cap, int* nlaunch) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op && B && nlaunch, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs && cap >= 0, "bad arguments");
    const slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    cudaStream_t st = h->h.stream;
    const size_t bytes = slu::hbs_solve_scratch_bytes(H, nrhs, sizeof(double));
    h->h.ws.reserve(bytes, st);
    double* scratch = h->h.ws.take<double>(bytes / sizeof(double));
    const size_t stride = ((sizeof(double) * (size_t)H.N * nrhs + 255) & ~size_t(255)) / 8;
    slu::LaunchTimes lt;
    lt.reserve(2 * (size_t)H.L);
    slu::enqueue_device_lead(st, 500);
    slu::ulv_solve_fused<double>(st, H, B, ldb, nrhs, scratch, stride, &lt);
    slu::stream_wait(st);
    const int n = (int)lt.level.size();
    *nlaunch = n;
    for (int k = 0; k < n && k < cap; ++k) {
      float ms = 0.f;
      SLU_CHECK_CUDA(cudaEventElapsedTime(&ms, lt.ev[2 * k], lt.ev[2 * k + 1]));
      if (ms_out) ms_out[k] = ms;
      if (level_out) level_out[k] = lt.level[k];
      if (kind_out) kind_out[k] = lt.kind[k];
    }
  });
}

int slu_ulv_autotune(slu_handle_t h, slu_hbs_t op, int nrhs, int precision, int reps,
                     int* knobs_out, int cap, int* nlaunch) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    SLU_REQUIRE(nrhs >= 1 && reps >= 1 && cap >= 0, "bad arguments");
    slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    slu::hbs_autotune_solve(h->h, H, nrhs, precision, reps);
    const std::vector<slu::PlanKnobs>& k = H.tuned[{precision, nrhs}];
    if (nlaunch) *nlaunch = (int)k.size();
    for (int i = 0; knobs_out && i < (int)k.size() && i < cap; ++i) {
      knobs_out[3 * i] = k[i].target;
      knobs_out[3 * i + 1] = k[i].rmin;
      knobs_out[3 * i + 2] = k[i].cmax;
    }
  });
}

int slu_hbs_set_null_space(slu_hbs_t op, int mode) {
  return guard(nullptr, [&] {
    SLU_REQUIRE(op, "null argument");
    SLU_REQUIRE(mode == 0 || mode == 1, "null-space mode must be 0 or 1");
    op->H.null_after_n = (mode == 1);
  });
}

int slu_hbs_info(slu_hbs_t op, int* L, int* N, int* levels, long long* NNvec, int* nsamples) {
  return guard(nullptr, [&] {
    SLU_REQUIRE(op, "null argument");
    const slu::Hbs& H = op->H;
    if (L) *L = H.L;
    if (N) *N = H.N;
    if (nsamples) *nsamples = H.nsamples;
    if (levels)
      for (int t = 0; t < H.L; ++t) {
        levels[4 * t + 0] = H.lv[t].Nb;
        levels[4 * t + 1] = H.lv[t].n;
        levels[4 * t + 2] = H.lv[t].k;
        levels[4 * t + 3] = H.lv[t].nu;
      }
    if (NNvec)
      for (size_t t = 0; t < H.NN.size(); ++t) NNvec[t] = H.NN[t];
  });
}

int slu_hbs_export(slu_handle_t h, slu_hbs_t op, int what, int level, double* dst, size_t count,
                   size_t* count_out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && op, "null argument");
    const slu::Hbs& H = op->H;
    SLU_REQUIRE(level >= 0 && level < H.L, "level out of range");
    const slu::Level& l = H.lv[level];
    const slu::DevBuf* b = nullptr;
    switch (what) {
      case 0: b = &l.U; break;
      case 1: b = &l.V; break;
      case 2: b = &l.D; break;
      case 3: b = &l.Q; break;
      case 4: b = &l.W; break;
      case 5: b = &l.R; break;
      case 6: b = &l.Uu; break;
      default: SLU_REQUIRE(false, "unknown factor id");
    }
    size_t n = b->bytes / 8;
    if (count_out) *count_out = n;
    if (dst && n) {
      SLU_REQUIRE(count >= n, "destination too small");
      SLU_CHECK_CUDA(cudaMemcpyAsync(dst, b->p, 8 * n, cudaMemcpyDeviceToDevice, h->h.stream));
    }
  });
}

int slu_hbs_nbytes(slu_hbs_t op, int which, size_t* out) {
  return guard(nullptr, [&] {
    SLU_REQUIRE(op && out, "null argument");
    *out = slu::hbs_nbytes(op->H, which);
  });
}

// ------------------------------------------------------------------ dense
int slu_lu_factor(slu_handle_t h, int n, double* A, int lda, long long sA, int* piv,
                  long long sP, int nb, int* info) {
  return guard(h, [&] {
    SLU_REQUIRE(h && A && piv, "null argument");
    SLU_REQUIRE(n >= 1 && lda >= n && nb >= 1, "bad shape");
    slu::lu_factor(h->h.stream, n, A, lda, sA, piv, sP, nb, info);
  });
}

int slu_lu_solve(slu_handle_t h, int trans, int n, const double* LU, int lda, long long sA,
                 const int* piv, long long sP, double* X, int ldx, long long sX, int nrhs,
                 int nb) {
  return guard(h, [&] {
    SLU_REQUIRE(h && LU && piv && X, "null argument");
    SLU_REQUIRE(n >= 1 && lda >= n && ldx >= nrhs && nb >= 1 && nrhs >= 1, "bad shape");
    slu::lu_solve<double>(h->h.stream, trans != 0, n, LU, lda, sA, piv, sP, X, ldx, sX, nrhs, nb);
  });
}

int slu_gemm_batched(slu_handle_t h, int transa, int transb, int M, int N, int K, double alpha,
                     const double* A, int lda, long long sA, const double* B, int ldb,
                     long long sB, double beta, double* C, int ldc, long long sC, int nb) {
  return guard(h, [&] {
    SLU_REQUIRE(h && A && B && C, "null argument");
    slu::gemm_batched<double>(h->h.stream, transa != 0, transb != 0, M, N, K, alpha, A, lda, sA,
                              0, B, ldb, sB, 0, beta, C, ldc, sC, 0, nb, 1);
  });
}

int slu_gemm_split3(slu_handle_t h, int M, int N, int K, double alpha, const double* A, int lda,
                    const double* B, int ldb, double beta, double* C, int ldc) {
  return guard(h, [&] {
    SLU_REQUIRE(h && A && B && C, "null argument");
    SLU_REQUIRE(M >= 0 && N >= 0 && K >= 1 && lda >= K && ldb >= N && ldc >= N, "bad shape");
    h->h.ws.reserve(slu::tc_gemm_workspace_bytes(M, N, K), h->h.stream);
    void* ws = h->h.ws.take<char>(slu::tc_gemm_workspace_bytes(M, N, K) - 256);
    slu::tc_gemm_split3(h->h.stream, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ws,
                        reinterpret_cast<unsigned int*>(h->h.info.as<int>()) + 1);
  });
}

// ------------------------------------------------------------------ tridiagonal
int slu_rb_factor(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                  const double* T, slu_rb_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && SiM && SiP && T && out, "null argument");
    auto p = std::make_unique<slu_dense_rb_s>();
    slu::rb_factor(h->h, p->S, nblk, m, SiM, SiP, T);
    *out = p.release();
  });
}

int slu_rb_factor_cyclic(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                         const double* T, slu_rb_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && SiM && SiP && T && out, "null argument");
    SLU_REQUIRE(nblk >= 2, "a periodic red-black system needs at least two blocks");
    auto p = std::make_unique<slu_dense_rb_s>();
    slu::rb_factor(h->h, p->S, nblk, m, SiM, SiP, T, false, true);
    *out = p.release();
  });
}

int slu_rb_solve_tc(slu_handle_t h, slu_rb_t rb, double* B, int ldb, int nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h && rb && B, "null argument");
    SLU_REQUIRE(!rb->thomas, "handle was made by slu_thomas_factor");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    slu::rb_solve(h->h, rb->S, B, ldb, nrhs, true);
  });
}

int slu_rb_factor_mixed(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                        const double* T, slu_rb_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && SiM && SiP && T && out, "null argument");
    auto p = std::make_unique<slu_dense_rb_s>();
    slu::rb_factor(h->h, p->S, nblk, m, SiM, SiP, T, true);
    *out = p.release();
  });
}

int slu_rb_refine(slu_handle_t h, slu_rb_t rb, const double* B, int ldb, double* X, int ldx,
                  int nrhs, double tol, int maxit, int* iters_out, double* relres_out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && rb && B && X, "null argument");
    SLU_REQUIRE(!rb->thomas, "handle was made by slu_thomas_factor");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs && ldx >= nrhs && maxit >= 1, "bad arguments");
    slu::rb_refine(h->h, rb->S, B, ldb, X, ldx, nrhs, tol, maxit, iters_out, relres_out);
  });
}

int slu_rb_solve(slu_handle_t h, slu_rb_t rb, double* B, int ldb, int nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h && rb && B, "null argument");
    SLU_REQUIRE(!rb->thomas, "handle was made by slu_thomas_factor");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    slu::rb_solve(h->h, rb->S, B, ldb, nrhs);
  });
}

int slu_rb_destroy(slu_rb_t rb) {
  return guard(nullptr, [&] { delete rb; });
}

int slu_thomas_factor(slu_handle_t h, int nblk, int m, const double* SiM, const double* SiP,
                      const double* T, slu_rb_t* out) {
  return guard(h, [&] {
    SLU_REQUIRE(h && SiM && SiP && T && out, "null argument");
    auto p = std::make_unique<slu_dense_rb_s>();
    p->thomas = true;
    slu::thomas_factor(h->h, p->S, nblk, m, SiM, SiP, T);
    *out = p.release();
  });
}

int slu_thomas_solve(slu_handle_t h, slu_rb_t th, double* B, int ldb, int nrhs) {
  return guard(h, [&] {
    SLU_REQUIRE(h && th && B, "null argument");
    SLU_REQUIRE(th->thomas, "handle was made by slu_rb_factor");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    slu::thomas_solve(h->h, th->S, B, ldb, nrhs);
  });
}

}  // extern "C"
