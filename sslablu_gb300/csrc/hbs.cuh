// HBS operator owned by the library: level factors, ULV factors, and the
// compression / factorisation / apply / solve drivers.
#pragma once
#include "dfloat.cuh"
#include "slablu_internal.cuh"

#include <mutex>

namespace slu {

// Per-call scratch arena (grow-only, stream ordered).
struct Workspace {
  DevBuf buf;
  size_t off = 0;
  void reset() { off = 0; }
  // Reserve `bytes` total for this call (reallocates if needed; contents lost).
  void reserve(size_t bytes, cudaStream_t st) {
    if (buf.bytes < bytes) buf.alloc(bytes + (bytes >> 2), st);
    off = 0;
  }
  template <class T> T* take(size_t count) {
    size_t b = (count * sizeof(T) + 255) & ~size_t(255);
    if (off + b > buf.bytes) throw Error(SLU_ERR_ALLOC, "workspace overflow");
    T* p = reinterpret_cast<T*>(reinterpret_cast<char*>(buf.p) + off);
    off += b;
    return p;
  }
};

// Pinned host memory for per-call uploads (task tables) and small read-backs
// (residual norms).  acquire() waits until the copy issued after the previous
// acquire has completed, so the buffer can be rewritten.
struct HostStage {
  char* p = nullptr;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
  HostStage() = default;
  HostStage(const HostStage&) = delete;
  HostStage& operator=(const HostStage&) = delete;
  ~HostStage() {
    if (done) cudaEventDestroy(done);
    if (p) cudaFreeHost(p);
  }
  char* acquire(size_t n) {
    if (done) SLU_CHECK_CUDA(cudaEventSynchronize(done));
    if (bytes < n) {
      if (p) SLU_CHECK_CUDA(cudaFreeHost(p));
      p = nullptr;
      bytes = 0;
      const size_t want = n + (n >> 2) + 4096;
      SLU_CHECK_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p), want));
      bytes = want;
    }
    return p;
  }
  // Marks the point on `st` after which the contents may be overwritten.
  void release(cudaStream_t st) {
    if (!done) SLU_CHECK_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    SLU_CHECK_CUDA(cudaEventRecord(done, st));
  }
};

struct Handle {
  cudaStream_t stream = nullptr;
  Workspace ws;
  HostStage upload, readback;
  DevBuf info;  // int[64] device status words
  std::string last_error;
};

// A step operator in the digit form of the tensor-core sweep (ozaki.cu):
// each row of every block scaled by its own power of two 2^E (max |row| <
// 2^E) and written as seven balanced base-256 digits, digit s a bfloat16
// value d * 2^(-8 s) (|d| <= 256, exact in bfloat16).  Per (block, row tile
// of NT rows, digit) one NT x wP image in the tcgen05 shared-memory core-
// matrix order (8 x 8 tiles of 128 bytes, K-major, no swizzle), so one bulk
// copy lands a digit slice ready for the MMA; rsc holds 2^E per row (0 for
// padding rows and zero rows).
struct OzOp {
  DevBuf dig, rsc;
  int Nb = 0, rows = 0, w = 0;
  int NT = 0, wP = 0, ntile = 0;
};

struct Level {
  int Nb = 0;   // blocks on this level
  int n = 0;    // rows (and columns of D) per block
  int k = 0;    // columns of U and V (0 on the root)
  int kU = 0;   // columns of the ULV Uu factor
  int nu = 0;   // rows of Ru per block (n - k; n on the root)
  int uu_rows = 0;  // rows of Uu per block
  DevBuf U, V, D;       // Nb*n x k, Nb*n x k, Nb*n x n
  DevBuf Q, W, R, Uu;   // Nb*n x n, Nb*n x n, Nb*nu x n, Nb*uu_rows x kU
  // single-precision copies of the solve factors (mixed-precision solve)
  DevBuf Uf, Df, Qf, Wf, Rf, Uuf;
  // step operators of the HBS apply (hbs_apply.cu), composed on first use:
  // mode N Aup = V^T, Adn = [D | U] per block (the root: D); mode T
  // AupT = U^T, AdnT = [D^T | V] (the root: D^T); Aupdf / Adndf: double-float
  // copies of the mode-N ones (the refinement residual)
  DevBuf Aup, Adn, AupT, AdnT, Aupdf, Adndf;
  // step operators of the mode-N solve (sweep_ops.cu): Qt = Q^T per block,
  // Sw = [G; H] per block (G only on the leaves; the root: [R^-1 Q^T; D R^-1 Q^T])
  DevBuf Qt, Sw;
  DevBuf Qtf, Swf;     // float32 copies
  // step operators of the mode-T solve: SwT = Sw^T per block, its columns
  // (the rows of Sw above the leaves) reordered to the children's [v; y]
  // ranges, child after child; the transposed forward steps use Q itself
  DevBuf SwT, SwTf;
  DevBuf Qtdf, Swdf;   // double-float copies (interleaved hi/lo pairs)
  // digit forms for the tensor-core (tcgen05) sweep and residual: Qt, Sw
  // (the root: Sw), Aup, Adn (the root: Adn)
  OzOp ozQt, ozSw, ozUp, ozDn;
  // and of the transposed solve and apply: Q, SwT (the root: SwT), AupT,
  // AdnT (the root: AdnT)
  OzOp ozQ, ozSwT, ozUpT, ozDnT;
};

struct RefinePlan;  // refine.cu: buffers + CUDA graphs of one refinement iteration

// Caps of a step launch plan (sweep_host.cuh plan_steps): the CTAs per SM a
// launch aims for, the row-slice floor it halves down to first, the widest
// column chunk.  The defaults serve untuned solves; hbs_autotune_solve picks
// them per step by timing.
struct PlanKnobs {
  int target = 2;
  int rmin = 16;
  int cmax = 64;
};

struct Hbs {
  int N = 0, L = 0, fac = 2;
  std::vector<Level> lv;           // lv[0] = leaves, lv[L-1] = root
  DevBuf perm;                     // int64[N]
  DevBuf iperm;                    // int64[N], iperm[perm[i]] = i
  // Top of the mode-N solve as one operator: the map from the vector entering
  // forward step `top` to the y and v vectors of backward step `top` (levels
  // top .. root), 2 N_top x N_top, composed at factor time from the steps it
  // replaces; -1 when the tree has no level of at most kTopRows rows below
  // the root's children.
  int top = -1;
  DevBuf Top, Topf, Topdf;
  bool identity_perm = true;
  std::vector<long long> NN;       // NNvec, L+1 entries
  bool has_mats = false, has_ulv = false, has_f32 = false, has_df = false, has_dfs = false;
  bool has_sweep = false;   // step operators composed (hbs_make_sweep)
  bool has_oz = false;      // digit forms for the tensor-core sweep (hbs_make_oz)
  bool has_ozT = false;     // ... of the transposed solve and apply (hbs_make_ozT)
  // apply operators, mode N / T (hbs_make_apply); composed on first use, so
  // set only after the composing stream has finished (other threads may read
  // them from their own streams right after)
  std::atomic<bool> has_apply[2] = {false, false};
  std::mutex lazy_mu;   // serialises first-use composition across threads
  // inner sweep of the mixed-precision refinement: 0 float32, 1 double-float,
  // 2 tensor-core digit sweep with a tensor-core digit residual (ozaki.cu)
  int refine_inner = 1;
  int rk = 0, nsamples = 0;
  // null space of a sketch block's Om^T used by compression: false takes the
  // last n columns of the complete Q (HBSnew.compute_UV), true every column
  // after the first n (HBStorch.compute_UV)
  bool null_after_n = false;
  // refinement plans per right-hand-side count; they capture factor pointers,
  // so every change of the factors clears them (invalidate_plans)
  std::map<int, std::shared_ptr<RefinePlan>> refine_plans;
  // tuned launch caps of the mode-N solve per (element type: 0 float64,
  // 1 float32, 2 double-float; right-hand-side count), one per launch;
  // dropped whenever the step operators are recomposed
  std::map<std::pair<int, int>, std::vector<PlanKnobs>> tuned;
  void invalidate_plans() { refine_plans.clear(); }
  // bumped whenever the step operators are recomposed: captured solve plans
  // hold their addresses and refuse to run after a change
  unsigned long long sweep_gen = 0;
  // expires with the operator (captured solve plans check it before running)
  std::shared_ptr<char> alive = std::make_shared<char>(0);
};

// One solve (mode N or T) captured as a CUDA graph for fixed right-hand-side
// and solution buffers, with its own scratch (ulv_solve.cu): a launch is one
// graph launch instead of one kernel launch per tree step.
struct SolvePlan {
  // the operators the graph reads (one; or every member of a grouped solve)
  std::vector<const Hbs*> H;
  std::vector<std::weak_ptr<char>> alive;
  std::vector<unsigned long long> gen;
  DevBuf scratch;
  cudaGraphExec_t exec = nullptr;
  long long kernels = 0;
  SolvePlan() = default;
  SolvePlan(const SolvePlan&) = delete;
  SolvePlan& operator=(const SolvePlan&) = delete;
  ~SolvePlan() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};
void solve_plan_create(Handle& h, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                       int c, bool trans, SolvePlan& P);
void solve_plan_launch(Handle& h, SolvePlan& P, bool wait);
// The grouped mode-N solve of hbs_solve_grouped (B[i] <- A_i^{-1} B[i]) for
// fixed blocks, captured once: step tables built and uploaded at creation.
void grouped_solve_plan_create(Handle& h, int count, Hbs* const* ops, double* const* B,
                               const int* ldb, const int* c, SolvePlan& P);

// A fixed sequence of grouped phases -- solves (kind 0, in place), applies
// (kind 1) and elementwise block operations (kinds 2-6: copy, zero, add,
// subtract, reverse subtract) -- with every table uploaded once and the
// whole sequence captured as one CUDA graph (group.cu).
void grouped_program_create(Handle& h, int nphase, const int* kind, const int* count,
                            Hbs* const* ops, double* const* X, double* const* Y,
                            const int* ld, const int* c, const long long* n, SolvePlan& P);

// The grouped mixed-precision refinement of hbs_refine_grouped for fixed
// blocks: buffers and task tables built once, an iteration replayed as CUDA
// graphs (group.cu).
struct GroupRefinePlan {
  std::vector<const Hbs*> H;
  std::vector<std::weak_ptr<char>> alive;
  std::vector<unsigned long long> gen;
  std::vector<int> idx;   // member index of each operator with columns
  int total = 0;          // members given (relres entries)
  virtual ~GroupRefinePlan() = default;
  virtual void run(Handle& h, double tol, int maxit, int* iters, double* relres) = 0;
};
std::unique_ptr<GroupRefinePlan> grouped_refine_plan_create(Handle& h, int count,
                                                            Hbs* const* ops, const double* const* B,
                                                            const int* ldb, double* const* X,
                                                            const int* ldx, const int* c);

// compression + interleaved ULV (HBSnew.HBSMAT.constructHBS_ULV)
void hbs_compress(Handle& h, Hbs& H, int Nb_leaf, int rk, int s, const double* Om,
                  const double* Psi, const double* Y, const double* Z, bool ulv);
// standalone ULV of loaded factors (ULVsparse.compute_ULV)
void hbs_factor(Handle& h, Hbs& H);
// u = A v (trans = false) or A^T v, caller ordering (through the tree permutation)
void hbs_apply(Handle& h, Hbs& H, bool trans, const double* X, int ldx, double* Yout,
               int ldy, int nrhs);
// ULV solve, reference semantics of HBSMAT.solve (with the permutation)
template <typename T>
void hbs_solve(Handle& h, const Hbs& H, bool trans, T* B, int ldb, int nrhs);
// The same solve with caller-provided scratch of hbs_solve_scratch_bytes()
// bytes (256-byte aligned); it makes no allocation of its own.
template <typename T>
void hbs_solve_scratch(cudaStream_t st, const Hbs& H, bool trans, T* B, int ldb, int nrhs,
                       T* scratch);
size_t hbs_solve_scratch_bytes(const Hbs& H, int nrhs, size_t elem);
// Device time of every launch of one fused solve (diagnostics): an event
// pair around each launch, with the launch's level and kind (0 forward,
// 1 root, 2 backward).
struct LaunchTimes {
  std::vector<cudaEvent_t> ev;
  std::vector<int> level, kind;
  LaunchTimes() = default;
  LaunchTimes(const LaunchTimes&) = delete;
  LaunchTimes& operator=(const LaunchTimes&) = delete;
  ~LaunchTimes() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
  }
  size_t next = 0;   // events are created up front (reserve), recorded in order
  void reserve(size_t launches) {
    while (ev.size() < 2 * launches) {
      cudaEvent_t e = nullptr;
      SLU_CHECK_CUDA(cudaEventCreate(&e));
      ev.push_back(e);
    }
  }
  void mark(cudaStream_t st) {
    if (next == ev.size()) reserve(ev.size() / 2 + 1);
    SLU_CHECK_CUDA(cudaEventRecord(ev[next++], st));
  }
  void done(int lvl, int k) {
    level.push_back(lvl);
    kind.push_back(k);
  }
};

// Mode-N solve with one fused kernel per level and sweep (ulv_solve.cu);
// scratch: five buffers of `stride` elements.  With X given, the right-hand
// sides are read from X (ld ldx) and B only receives the solution.
template <typename T>
void ulv_solve_fused(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch,
                     size_t stride, LaunchTimes* times = nullptr, const T* X = nullptr,
                     int ldx = 0);
// Mode-T solve B <- A^{-T} B (reading X when given) with the transposed
// step operators; scratch as ulv_solve_fused.
template <typename T>
void ulv_solve_T(cudaStream_t st, const Hbs& H, T* B, int ldb, int c, T* scratch, size_t stride,
                 const T* X = nullptr, int ldx = 0);
// Times every launch of the mode-N solve for `c` right-hand sides under a set
// of plan caps and keeps the fastest per launch (H.tuned); precision 0
// float64, 2 double-float.  Results are unchanged: the caps only move work
// between CTAs, never the order of a dot product's terms.
void hbs_autotune_solve(Handle& h, Hbs& H, int c, int precision, int reps);
// Enqueues a kernel that only sleeps for about `us` microseconds (a fixed
// number of __nanosleep calls, no waiting on anything), so that the host can
// queue the launches that follow before the device reaches them: their event
// timestamps then measure device time, not host enqueue gaps.
void enqueue_device_lead(cudaStream_t st, int us);
// Apply as step kernels (hbs_apply.cu): scratch of hbs_apply_scratch_elems
// elements of T; the operators of the direction must have been composed
// (hbs_make_apply; for T = dfloat, hbs_make_df).
size_t hbs_apply_scratch_elems(const Hbs& H, int c);
void hbs_make_apply(Handle& h, Hbs& H, bool trans);
template <typename T>
void hbs_apply_fused(cudaStream_t st, const Hbs& H, bool trans, const T* X, int ldx, T* Y,
                     int ldy, int c, T* scratch);
void hbs_make_f32(Handle& h, Hbs& H);
// Composes the step operators of the mode-N solve from the ULV factors.
void hbs_make_sweep(Handle& h, Hbs& H);
// Double-float copies of the step operators (dfloat ULV sweep).
void hbs_make_dfs(Handle& h, Hbs& H);
// B (N x c float64, caller ordering) <- A^{-1} B with the double-float sweep;
// scratch of hbs_solve_df_scratch_bytes() bytes.
size_t hbs_solve_df_scratch_bytes(const Hbs& H, int c);
void hbs_solve_df(cudaStream_t st, const Hbs& H, double* B, int ldb, int c, void* scratch);
// Mixed-precision refinement replayed as CUDA graphs (refine.cu).
void hbs_refine(Handle& h, Hbs& H, const double* B, int ldb, double* X, int ldx, int c,
                double tol, int maxit, int* iters, double* relres);
// Double-float apply Y = A X (mode N; float64 in and out, double-float
// arithmetic): the mode-N apply operators split once by hbs_make_df.
void hbs_make_df(Handle& h, Hbs& H);
size_t hbs_apply_df_scratch_bytes(const Hbs& H, int c);
void hbs_apply_df(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch);
size_t hbs_nbytes(const Hbs& H, int which);

// ---------------------------------------------------------------- tensor-core sweep
// (ozaki.cu) Digit forms of the mode-N solve and apply step operators, and the
// solve / apply run as tcgen05 block products of bfloat16 digits with exact
// float32 accumulation.  Vectors between steps are double-float pairs.
void hbs_make_oz(Handle& h, Hbs& H);
// The digit forms of the transposed (mode T) solve and apply operators.
void hbs_make_ozT(Handle& h, Hbs& H);
// Scratch (bytes) of ulv_solve_oz / hbs_apply_oz for c right-hand sides.
size_t hbs_oz_scratch_bytes(const Hbs& H, int c);
// Y <- A^{-1} X (mode N) and Y <- A X on the tensor cores; X, Y N x c
// float64 (distinct buffers), scratch of hbs_oz_scratch_bytes bytes; err a
// device word set on a device wait timeout.
void ulv_solve_oz(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch, unsigned* err);
// Y <- A^{-T} X on the tensor cores (the transposed steps of the float64
// mode-T solve, caller ordering through the inverse permutation).
void ulv_solve_oz_T(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y,
                    int ldy, int c, void* scratch, unsigned* err);
// With resb (N x c, leading dimension ldy) the apply returns the residual
// Y = resb - A X instead, and rnorm2 (c entries, zeroed by the caller)
// accumulates its squared column norms.
void hbs_apply_oz(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch, unsigned* err, const double* resb = nullptr,
                  double* rnorm2 = nullptr, bool trans = false);

// Factor pointers of one level by arithmetic type (float64 factors or their
// float32 copies).
template <typename T>
struct FacPtr;
template <>
struct FacPtr<double> {
  static const double* U(const Level& l) { return l.U.as<double>(); }
  static const double* D(const Level& l) { return l.D.as<double>(); }
  static const double* Q(const Level& l) { return l.Q.as<double>(); }
  static const double* W(const Level& l) { return l.W.as<double>(); }
  static const double* R(const Level& l) { return l.R.as<double>(); }
  static const double* Uu(const Level& l) { return l.Uu.as<double>(); }
  static const double* Qt(const Level& l) { return l.Qt.as<double>(); }
  static const double* Sw(const Level& l) { return l.Sw.as<double>(); }
  static const double* SwT(const Level& l) { return l.SwT.as<double>(); }
  static const double* Top(const Hbs& H) { return H.Top.as<double>(); }
};
template <>
struct FacPtr<float> {
  static const float* U(const Level& l) { return l.Uf.as<float>(); }
  static const float* D(const Level& l) { return l.Df.as<float>(); }
  static const float* Q(const Level& l) { return l.Qf.as<float>(); }
  static const float* W(const Level& l) { return l.Wf.as<float>(); }
  static const float* R(const Level& l) { return l.Rf.as<float>(); }
  static const float* Uu(const Level& l) { return l.Uuf.as<float>(); }
  static const float* Qt(const Level& l) { return l.Qtf.as<float>(); }
  static const float* Sw(const Level& l) { return l.Swf.as<float>(); }
  static const float* SwT(const Level& l) { return l.SwTf.as<float>(); }
  static const float* Top(const Hbs& H) { return H.Topf.as<float>(); }
};

template <>
struct FacPtr<dfloat> {
  static const dfloat* Qt(const Level& l) { return l.Qtdf.as<dfloat>(); }
  static const dfloat* Sw(const Level& l) { return l.Swdf.as<dfloat>(); }
  static const dfloat* Top(const Hbs& H) { return H.Topdf.as<dfloat>(); }
  // the transposed steps run on the tensor cores only (their digit forms,
  // ozSwT / ozQ): no double-float copies of Q or SwT exist
  static const dfloat* Q(const Level&) { return nullptr; }
  static const dfloat* SwT(const Level&) { return nullptr; }
};

// Grouped solves over many operators (group.cu): one launch per tree step for
// the whole group.  B[i] is N_i x c[i] row-major with leading dimension ldb[i].
// Grouped apply Y[i] = A_i X[i] (trans[i] = 0) or A_i^T X[i]: one launch per
// tree step for the whole group.
void hbs_apply_grouped(Handle& h, int count, Hbs* const* ops, const int* trans,
                       const double* const* X, const int* ldx, double* const* Y, const int* ldy,
                       const int* c);
void hbs_solve_grouped(Handle& h, int count, Hbs* const* ops, double* const* B, const int* ldb,
                       const int* c);
// Mixed-precision refinement of the group; iters is the common iteration
// count, relres[i] the worst column residual of member i.
void hbs_refine_grouped(Handle& h, int count, Hbs* const* ops, const double* const* B,
                        const int* ldb, double* const* X, const int* ldx, const int* c,
                        double tol, int maxit, int* iters, double* relres);

}  // namespace slu
