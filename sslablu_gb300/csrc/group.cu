// Grouped HBS solves: many operators of uneven sizes, one launch per tree step.
//
// The reference solves one operator per call (HBSnew.HBSMAT.solve,
// matAssembly/HBS/HBSnew.py:393-416, through ULVsparse.solve,
// matAssembly/HBS/ULVsparse.py:296-327); the slab solvers call it for every
// block of every level.  Solving a group of operators with the per-operator
// kernels costs up to 2L-1 launches per operator, each too small to fill 152 SMs.
// Here each tree step of every member becomes a *segment* of one launch: a
// task table lists, per segment, the member's factors, buffers and column
// chunking, and the CTA range it owns; a CTA finds its segment by binary
// search over the range starts and runs the same device body as the
// per-operator kernel (sweep.cuh).  The schedule is
//   forward  t = 0 .. maxL-2   (members with L_i >= t + 2)
//   root                         (every member)
//   backward t = maxL-2 .. 0   (members with L_i >= t + 2)
// so members of different depths share launches, and each member's own
// sequence of steps (and of ping-pong buffers) is exactly its solo sequence.
//
// Mixed-precision refinement of a group (hbs_refine_grouped) runs the same
// loop as refine.cu over concatenated buffers: one launch per elementwise step
// for the whole group, the grouped inner sweep (double-float, or float32 when
// every member asks for it), the grouped double-float apply (the apply steps
// of hbs_apply.cu on float32 pairs), and segmented column norms.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "hbs.cuh"
#include "refine_kernels.cuh"
#include "sweep_host.cuh"

namespace slu {
namespace {

// One tree step of one member in a grouped ULV sweep: its step (sweep.cuh),
// the first CTA of its range and its column chunks per row slice.
template <typename T>
struct StepSeg {
  sweep::Step<T> s;
  int cta0, ncch;
};

struct ColSeg {  // one right-hand-side column of a concatenated buffer
  long long off;
  int rows, ld;
};

struct CopySeg {  // one member's rows x cols block between two layouts
  const double* src;
  double* dst;
  int lds, ldd, rows, cols;
};

template <class S>
__device__ __forceinline__ int find_seg(const S* __restrict__ segs, int nseg) {
  int lo = 0, hi = nseg - 1;
  const int x = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].cta0 <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <typename T>
__global__ void __launch_bounds__(sweep::kMaxThreads)
group_step_kernel(const StepSeg<T>* __restrict__ segs, int nseg) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const StepSeg<T>& g = segs[find_seg(segs, nseg)];
  const int local = blockIdx.x - g.cta0;
  sweep::step_body<T>(g.s, sm_raw, local / g.ncch, local - (local / g.ncch) * g.ncch);
}

// out[j] = sum_i A[cols[j].off + i * cols[j].ld]^2
__global__ void colnorm_seg_k(const ColSeg* __restrict__ cols, const double* __restrict__ A,
                              double* __restrict__ out) {
  const ColSeg s = cols[blockIdx.x];
  double acc = 0.0;
  for (int i = threadIdx.x; i < s.rows; i += blockDim.x) {
    const double v = A[s.off + (long long)i * s.ld];
    acc += v * v;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    out[blockIdx.x] = t;
  }
}

__global__ void seg_copy_k(const CopySeg* __restrict__ segs) {
  const CopySeg s = segs[blockIdx.x];
  const long long n = (long long)s.rows * s.cols;
  for (long long e = (long long)blockIdx.y * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.y * blockDim.x) {
    const long long i = e / s.cols, j = e - i * s.cols;
    s.dst[i * s.ldd + j] = s.src[i * s.lds + j];
  }
}

// One contiguous block of an elementwise phase of a grouped program.
struct EwSeg {
  const double* x;
  double* y;
  long long n;
  int kind;   // 2 copy y = x, 3 zero y = 0, 4 add y += x, 5 sub y -= x, 6 rsub y = x - y
};

__global__ void ew_seg_k(const EwSeg* __restrict__ segs) {
  const EwSeg s = segs[blockIdx.x];
  for (long long e = (long long)blockIdx.y * blockDim.x + threadIdx.x; e < s.n;
       e += (long long)gridDim.y * blockDim.x) {
    switch (s.kind) {
      case 2: s.y[e] = s.x[e]; break;
      case 3: s.y[e] = 0.0; break;
      case 4: s.y[e] = s.y[e] + s.x[e]; break;
      case 5: s.y[e] = s.y[e] - s.x[e]; break;
      default: s.y[e] = s.x[e] - s.y[e]; break;
    }
  }
}

// ------------------------------------------------------------------ host side
// Per-member device buffers of a grouped ULV sweep (five of `stride`).
template <typename T>
struct SolveBufs {
  T* ru;
  T* P[4];
};

// Step tables of a grouped sweep: the segments of every launch, back to back.
template <typename T>
struct StepTable {
  std::vector<StepSeg<T>> segs;
  std::vector<int> off, cnt;
  std::vector<sweep::LaunchPlan> plan;
  void add(std::vector<sweep::Step<T>>& v) {
    if (v.empty()) return;
    std::vector<sweep::Step<T>*> ptr;
    for (auto& x : v) ptr.push_back(&x);
    const sweep::LaunchPlan p = sweep::plan_steps(ptr.data(), (int)ptr.size());
    off.push_back((int)segs.size());
    cnt.push_back((int)v.size());
    plan.push_back(p);
    long long cta = 0;
    for (auto& x : v) {
      StepSeg<T> g{};
      g.s = x;
      g.ncch = (x.c + x.cpb - 1) / x.cpb;
      g.cta0 = (int)cta;
      cta += (long long)x.nb * x.nrch * g.ncch;
      segs.push_back(g);
    }
  }
};

// Builds the step tables of a grouped mode-N ULV sweep; B[i] is solved in
// place.  Member i runs exactly its solo sequence of steps and buffers.
template <typename T>
void build_solve(const std::vector<const Hbs*>& H, const std::vector<int>& c,
                 const std::vector<T*>& B, const std::vector<int>& ldb,
                 const std::vector<SolveBufs<T>>& buf, StepTable<T>& tab) {
  const int m = (int)H.size();
  int maxL = 0;
  for (int i = 0; i < m; ++i) maxL = std::max(maxL, sweep::chain_levels(*H[i]));
  std::vector<sweep::Step<T>> v;
  for (int t = 0; t + 1 < maxL; ++t) {
    v.clear();
    for (int i = 0; i < m; ++i) {
      if (sweep::chain_levels(*H[i]) < t + 2) continue;
      v.push_back(sweep::forward_step<T>(
          *H[i], t, t == 0 ? B[i] : buf[i].P[(t - 1) & 1], t == 0 ? ldb[i] : c[i],
          t == 0 ? H[i]->perm.as<int64_t>() : nullptr, buf[i].ru + H[i]->NN[t] * c[i],
          buf[i].P[t & 1], c[i]));
    }
    tab.add(v);
  }
  v.clear();
  for (int i = 0; i < m; ++i) {
    const int L = sweep::chain_levels(*H[i]);
    if (H[i]->top >= 1)
      v.push_back(sweep::top_step<T>(*H[i], buf[i].P[(L - 2) & 1], c[i], buf[i].P[2],
                                     buf[i].P[3], c[i]));
    else
      v.push_back(sweep::root_step<T>(*H[i], L == 1 ? B[i] : buf[i].P[(L - 2) & 1],
                                      L == 1 ? ldb[i] : c[i], B[i], ldb[i], buf[i].P[2],
                                      buf[i].P[3], c[i]));
  }
  tab.add(v);
  for (int t = maxL - 2; t >= 0; --t) {
    v.clear();
    for (int i = 0; i < m; ++i) {
      const int L = sweep::chain_levels(*H[i]);
      if (L < t + 2) continue;
      const int in = ((L - 2 - t) % 2 == 0) ? 2 : 0, out = in == 2 ? 0 : 2;
      v.push_back(sweep::backward_step<T>(*H[i], t, buf[i].ru + H[i]->NN[t] * c[i],
                                          buf[i].P[in + 1], buf[i].P[in], buf[i].P[out],
                                          buf[i].P[out + 1], B[i], ldb[i], c[i]));
    }
    tab.add(v);
  }
}

// Per-member buffers of a grouped apply: VV[t] for t >= 1 and u[2]
// (hbs_apply_scratch_elems elements).
template <typename T>
struct ApplyBufs {
  std::vector<T*> VV;
  T* u[2];
};

template <typename T>
ApplyBufs<T> carve_apply(const Hbs& H, int c, T* base) {
  ApplyBufs<T> d;
  d.VV.assign(H.L, nullptr);
  size_t off = 0;
  for (int t = 0; t + 1 < H.L; ++t) {
    d.VV[t + 1] = base + off;
    off += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 63) & ~size_t(63);
  }
  d.u[0] = base + off;
  d.u[1] = base + off + (((size_t)H.N * c + 63) & ~size_t(63));
  return d;
}

// Step tables of a grouped double-float apply Y[i] = A_i X[i] (the steps of
// hbs_apply_fused, tree-step by tree-step across members).
void build_apply_df(const std::vector<const Hbs*>& H, const std::vector<int>& c,
                    const std::vector<const dfloat*>& X, const std::vector<dfloat*>& Y,
                    const std::vector<ApplyBufs<dfloat>>& buf, StepTable<dfloat>& tab) {
  const int m = (int)H.size();
  int maxL = 0;
  for (int i = 0; i < m; ++i) maxL = std::max(maxL, H[i]->L);
  std::vector<sweep::Step<dfloat>> v;
  for (int t = 0; t + 1 < maxL; ++t) {
    v.clear();
    for (int i = 0; i < m; ++i) {
      if (H[i]->L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      v.push_back(sweep::up_step<dfloat>(l, l.Aupdf.as<dfloat>(), t == 0 ? X[i] : buf[i].VV[t],
                                         c[i], t == 0 ? H[i]->perm.as<int64_t>() : nullptr,
                                         buf[i].VV[t + 1], c[i]));
    }
    tab.add(v);
  }
  v.clear();
  for (int i = 0; i < m; ++i) {
    const int L = H[i]->L;
    const Level& r = H[i]->lv[L - 1];
    const int64_t* perm = H[i]->perm.as<int64_t>();
    if (L == 1)
      v.push_back(sweep::down_step<dfloat>(r, r.Adndf.as<dfloat>(), true, X[i], c[i], perm,
                                           nullptr, Y[i], c[i], perm, c[i]));
    else
      v.push_back(sweep::down_step<dfloat>(r, r.Adndf.as<dfloat>(), true, buf[i].VV[L - 1], c[i],
                                           nullptr, nullptr, buf[i].u[0], c[i], nullptr, c[i]));
  }
  tab.add(v);
  for (int t = maxL - 2; t >= 0; --t) {
    v.clear();
    for (int i = 0; i < m; ++i) {
      const int L = H[i]->L;
      if (L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      const int cur = (L - 2 - t) & 1;
      const bool leaf = t == 0;
      const int64_t* perm = leaf ? H[i]->perm.as<int64_t>() : nullptr;
      v.push_back(sweep::down_step<dfloat>(l, l.Adndf.as<dfloat>(), false,
                                           leaf ? X[i] : buf[i].VV[t], c[i], perm, buf[i].u[cur],
                                           leaf ? Y[i] : buf[i].u[cur ^ 1], c[i], perm, c[i]));
    }
    tab.add(v);
  }
}

template <typename T>
void launch_solve(cudaStream_t st, const StepTable<T>& tab, const StepSeg<T>* dsegs) {
  auto kern = group_step_kernel<T>;
  for (size_t i = 0; i < tab.plan.size(); ++i) {
    const sweep::LaunchPlan& p = tab.plan[i];
    if (p.ctas == 0) continue;
    ensure_smem(reinterpret_cast<const void*>(kern), p.smem);
    sweep::launch_pdl(kern, p, st, "group_step_kernel", dsegs + tab.off[i], tab.cnt[i]);
  }
}

// Sizes of device regions taken in order from the workspace.
struct Plan {
  std::vector<size_t> bytes;
  size_t add(size_t b) {
    bytes.push_back(b);
    return bytes.size() - 1;
  }
  size_t total() const {
    size_t t = 0;
    for (size_t b : bytes) t += (b + 255) & ~size_t(255);
    return t;
  }
};

// Table blob: appended host arrays, uploaded in one copy.
struct Blob {
  std::vector<char> host;
  template <class S>
  size_t put(const std::vector<S>& v) {
    const size_t at = (host.size() + 255) & ~size_t(255);
    host.resize(at + v.size() * sizeof(S));
    if (!v.empty()) std::memcpy(host.data() + at, v.data(), v.size() * sizeof(S));
    return at;
  }
};

void upload(Handle& h, const Blob& b, void* dev) {
  if (b.host.empty()) return;
  char* p = h.upload.acquire(b.host.size());
  std::memcpy(p, b.host.data(), b.host.size());
  SLU_CHECK_CUDA(cudaMemcpyAsync(dev, p, b.host.size(), cudaMemcpyHostToDevice, h.stream));
  h.upload.release(h.stream);
}

size_t blob_bound(size_t payload, int arrays) { return payload + 256 * (size_t)(arrays + 1); }

inline size_t round64(size_t n) { return (n + 63) & ~size_t(63); }

// Step tables of a grouped float64 apply Y[i] = op_i(A_i) X[i] (mode N or T
// per member; the steps of hbs_apply_fused, tree step by tree step).
void build_apply64(const std::vector<const Hbs*>& H, const std::vector<int>& tr,
                   const std::vector<int>& c, const std::vector<const double*>& X,
                   const std::vector<int>& ldx, const std::vector<double*>& Y,
                   const std::vector<int>& ldy, const std::vector<ApplyBufs<double>>& buf,
                   StepTable<double>& tab) {
  const int m = (int)H.size();
  int maxL = 0;
  for (int i = 0; i < m; ++i) maxL = std::max(maxL, H[i]->L);
  auto up = [&](const Level& l, int i) { return (tr[i] ? l.AupT : l.Aup).as<double>(); };
  auto dn = [&](const Level& l, int i) { return (tr[i] ? l.AdnT : l.Adn).as<double>(); };
  std::vector<sweep::Step<double>> v;
  for (int t = 0; t + 1 < maxL; ++t) {
    v.clear();
    for (int i = 0; i < m; ++i) {
      if (H[i]->L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      v.push_back(sweep::up_step<double>(l, up(l, i), t == 0 ? X[i] : buf[i].VV[t],
                                         t == 0 ? ldx[i] : c[i],
                                         t == 0 ? H[i]->perm.as<int64_t>() : nullptr,
                                         buf[i].VV[t + 1], c[i]));
    }
    tab.add(v);
  }
  v.clear();
  for (int i = 0; i < m; ++i) {
    const int L = H[i]->L;
    const Level& r = H[i]->lv[L - 1];
    const int64_t* perm = H[i]->perm.as<int64_t>();
    if (L == 1)
      v.push_back(sweep::down_step<double>(r, dn(r, i), true, X[i], ldx[i], perm, nullptr, Y[i],
                                           ldy[i], perm, c[i]));
    else
      v.push_back(sweep::down_step<double>(r, dn(r, i), true, buf[i].VV[L - 1], c[i], nullptr,
                                           nullptr, buf[i].u[0], c[i], nullptr, c[i]));
  }
  tab.add(v);
  for (int t = maxL - 2; t >= 0; --t) {
    v.clear();
    for (int i = 0; i < m; ++i) {
      const int L = H[i]->L;
      if (L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      const int cur = (L - 2 - t) & 1;
      const bool leaf = t == 0;
      const int64_t* perm = leaf ? H[i]->perm.as<int64_t>() : nullptr;
      v.push_back(sweep::down_step<double>(l, dn(l, i), false, leaf ? X[i] : buf[i].VV[t],
                                           leaf ? ldx[i] : c[i], perm, buf[i].u[cur],
                                           leaf ? Y[i] : buf[i].u[cur ^ 1], leaf ? ldy[i] : c[i],
                                           perm, c[i]));
    }
    tab.add(v);
  }
}

}  // namespace

void hbs_solve_grouped(Handle& h, int count, Hbs* const* ops, double* const* B, const int* ldb,
                       const int* c) {
  SLU_REQUIRE(count >= 0 && (count == 0 || (ops && B && ldb && c)), "null argument");
  std::vector<const Hbs*> H;
  std::vector<double*> Bm;
  std::vector<int> cm, ldm;
  for (int i = 0; i < count; ++i) {
    SLU_REQUIRE(ops[i], "null operator");
    SLU_REQUIRE(c[i] >= 0, "bad right-hand-side count");
    if (c[i] == 0) continue;
    SLU_REQUIRE(B[i] && ldb[i] >= c[i], "bad right-hand side");
    SLU_REQUIRE(ops[i]->has_ulv, "ULV factors not computed");
    H.push_back(ops[i]);
    Bm.push_back(B[i]);
    cm.push_back(c[i]);
    ldm.push_back(ldb[i]);
  }
  const int m = (int)H.size();
  if (m == 0) return;
  cudaStream_t st = h.stream;
  // device regions: the task table, then five buffers per member
  size_t nseg = 0;
  for (const Hbs* x : H) nseg += 2 * (size_t)x->L;
  Plan plan;
  plan.add(blob_bound(nseg * sizeof(StepSeg<double>), 1));
  std::vector<size_t> stride(m);
  for (int i = 0; i < m; ++i) {
    stride[i] = round64((size_t)H[i]->N * cm[i]);
    plan.add(5 * stride[i] * sizeof(double));
  }
  h.ws.reserve(plan.total(), st);
  char* dtab = h.ws.take<char>(plan.bytes[0]);
  std::vector<SolveBufs<double>> buf(m);
  for (int i = 0; i < m; ++i) {
    double* s = h.ws.take<double>(5 * stride[i]);
    buf[i].ru = s;
    for (int j = 0; j < 4; ++j) buf[i].P[j] = s + (j + 1) * stride[i];
  }
  StepTable<double> steps;
  build_solve<double>(H, cm, Bm, ldm, buf, steps);
  Blob blob;
  const size_t at = blob.put(steps.segs);
  SLU_REQUIRE(blob.host.size() <= plan.bytes[0], "task table overflow");
  upload(h, blob, dtab);
  launch_solve<double>(st, steps, reinterpret_cast<const StepSeg<double>*>(dtab + at));
}

void grouped_solve_plan_create(Handle& h, int count, Hbs* const* ops, double* const* B,
                               const int* ldb, const int* c, SolvePlan& P) {
  SLU_REQUIRE(count >= 0 && (count == 0 || (ops && B && ldb && c)), "null argument");
  std::vector<const Hbs*> H;
  std::vector<double*> Bm;
  std::vector<int> cm, ldm;
  for (int i = 0; i < count; ++i) {
    SLU_REQUIRE(ops[i], "null operator");
    SLU_REQUIRE(c[i] >= 0, "bad right-hand-side count");
    if (c[i] == 0) continue;
    SLU_REQUIRE(B[i] && ldb[i] >= c[i], "bad right-hand side");
    SLU_REQUIRE(ops[i]->has_ulv && ops[i]->has_sweep, "ULV factors not computed");
    H.push_back(ops[i]);
    Bm.push_back(B[i]);
    cm.push_back(c[i]);
    ldm.push_back(ldb[i]);
  }
  const int m = (int)H.size();
  for (const Hbs* x : H) {
    P.H.push_back(x);
    P.alive.push_back(x->alive);
    P.gen.push_back(x->sweep_gen);
  }
  if (m == 0) return;
  cudaStream_t st = h.stream;
  // plan-owned device regions: the task table, then five buffers per member
  size_t nseg = 0;
  for (const Hbs* x : H) nseg += 2 * (size_t)x->L;
  Plan plan;
  plan.add(blob_bound(nseg * sizeof(StepSeg<double>), 1));
  std::vector<size_t> stride(m);
  for (int i = 0; i < m; ++i) {
    stride[i] = round64((size_t)H[i]->N * cm[i]);
    plan.add(5 * stride[i] * sizeof(double));
  }
  P.scratch.alloc(plan.total(), st);
  char* base = static_cast<char*>(P.scratch.p);
  char* dtab = base;
  size_t off = (plan.bytes[0] + 255) & ~size_t(255);
  std::vector<SolveBufs<double>> buf(m);
  for (int i = 0; i < m; ++i) {
    double* s = reinterpret_cast<double*>(base + off);
    buf[i].ru = s;
    for (int j = 0; j < 4; ++j) buf[i].P[j] = s + (j + 1) * stride[i];
    off += (5 * stride[i] * sizeof(double) + 255) & ~size_t(255);
  }
  StepTable<double> steps;
  build_solve<double>(H, cm, Bm, ldm, buf, steps);
  Blob blob;
  const size_t at = blob.put(steps.segs);
  SLU_REQUIRE(blob.host.size() <= plan.bytes[0], "task table overflow");
  upload(h, blob, dtab);
  auto kern = group_step_kernel<double>;
  for (const sweep::LaunchPlan& p : steps.plan)
    if (p.ctas > 0) ensure_smem(reinterpret_cast<const void*>(kern), p.smem);
  stream_wait(st);   // table and buffers in place before the capture
  cudaStream_t cs = nullptr;
  SLU_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  const long long n0 = launch_thread();
  try {
    SLU_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
      launch_solve<double>(cs, steps, reinterpret_cast<const StepSeg<double>*>(dtab + at));
    } catch (...) {
      cudaStreamEndCapture(cs, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    SLU_CHECK_CUDA(cudaStreamEndCapture(cs, &g));
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
}

void grouped_program_create(Handle& h, int nphase, const int* kind, const int* count,
                            Hbs* const* ops, double* const* X, double* const* Y,
                            const int* ld, const int* c, const long long* n, SolvePlan& P) {
  SLU_REQUIRE(nphase >= 0 && (nphase == 0 || (kind && count)), "null argument");
  cudaStream_t st = h.stream;
  // pass 1: members of every phase, tables and the scratch each phase needs
  struct Phase {
    int kind;
    std::vector<const Hbs*> H;
    std::vector<int> cm, ldm, tr;
    std::vector<double*> Xm, Ym;
    std::vector<const double*> Xc;
    std::vector<EwSeg> ew;
    size_t scratch = 0;
  };
  std::vector<Phase> ph(nphase);
  long long at = 0;
  size_t nseg_total = 0, scratch_max = 0;
  for (int p = 0; p < nphase; ++p) {
    Phase& f = ph[p];
    f.kind = kind[p];
    SLU_REQUIRE(f.kind >= 0 && f.kind <= 6, "unknown grouped program phase");
    SLU_REQUIRE(count[p] >= 0, "bad phase size");
    for (int q = 0; q < count[p]; ++q, ++at) {
      if (f.kind <= 1) {
        SLU_REQUIRE(ops && ops[at] && X && X[at] && ld && c, "null argument");
        SLU_REQUIRE(c[at] >= 1 && ld[at] >= c[at], "bad right-hand side");
        Hbs& Hq = *ops[at];
        if (f.kind == 0) {
          SLU_REQUIRE(Hq.has_ulv && Hq.has_sweep, "ULV factors not computed");
        } else {
          SLU_REQUIRE(Y && Y[at], "null argument");
          SLU_REQUIRE(Hq.has_mats, "HBS factors not loaded");
          if (!Hq.has_apply[0]) {
            std::lock_guard<std::mutex> lock(Hq.lazy_mu);
            if (!Hq.has_apply[0]) hbs_make_apply(h, Hq, false);
          }
          f.Ym.push_back(Y[at]);
          f.Xc.push_back(X[at]);
          f.tr.push_back(0);
        }
        f.H.push_back(&Hq);
        f.Xm.push_back(X[at]);
        f.cm.push_back(c[at]);
        f.ldm.push_back(ld[at]);
      } else {
        SLU_REQUIRE(n && n[at] >= 0 && Y && Y[at] && (f.kind == 3 || (X && X[at])),
                    "bad elementwise block");
        f.ew.push_back(EwSeg{f.kind == 3 ? nullptr : X[at], Y[at], n[at], f.kind});
      }
    }
    for (size_t i = 0; i < f.H.size(); ++i) {
      if (f.kind == 0) f.scratch += (5 * round64((size_t)f.H[i]->N * f.cm[i]) * 8 + 255) & ~size_t(255);
      else f.scratch += (8 * hbs_apply_scratch_elems(*f.H[i], f.cm[i]) + 255) & ~size_t(255);
      nseg_total += 2 * (size_t)f.H[i]->L;
    }
    nseg_total += f.ew.size();
    scratch_max = std::max(scratch_max, f.scratch);
    for (const Hbs* x : f.H) {
      P.H.push_back(x);
      P.alive.push_back(x->alive);
      P.gen.push_back(x->sweep_gen);
    }
  }
  // device memory: all tables (uploaded once), then one scratch region the
  // phases share (they run one after another)
  const size_t tab_bytes = blob_bound(nseg_total * std::max(sizeof(StepSeg<double>),
                                                            sizeof(EwSeg)), 2 * nphase + 1);
  P.scratch.alloc(tab_bytes + scratch_max + 512, st);
  char* dtab = static_cast<char*>(P.scratch.p);
  char* dscr = dtab + ((tab_bytes + 255) & ~size_t(255));
  Blob blob;
  std::vector<StepTable<double>> tabs(nphase);
  std::vector<size_t> tab_at(nphase, 0);
  for (int p = 0; p < nphase; ++p) {
    Phase& f = ph[p];
    if (f.kind >= 2) {
      if (!f.ew.empty()) tab_at[p] = blob.put(f.ew);
      continue;
    }
    if (f.H.empty()) continue;
    size_t off = 0;
    if (f.kind == 0) {
      std::vector<SolveBufs<double>> buf(f.H.size());
      for (size_t i = 0; i < f.H.size(); ++i) {
        const size_t stride = round64((size_t)f.H[i]->N * f.cm[i]);
        double* sb = reinterpret_cast<double*>(dscr + off);
        buf[i].ru = sb;
        for (int j = 0; j < 4; ++j) buf[i].P[j] = sb + (j + 1) * stride;
        off += (5 * stride * 8 + 255) & ~size_t(255);
      }
      build_solve<double>(f.H, f.cm, f.Xm, f.ldm, buf, tabs[p]);
    } else {
      std::vector<ApplyBufs<double>> buf(f.H.size());
      for (size_t i = 0; i < f.H.size(); ++i) {
        buf[i] = carve_apply(*f.H[i], f.cm[i], reinterpret_cast<double*>(dscr + off));
        off += (8 * hbs_apply_scratch_elems(*f.H[i], f.cm[i]) + 255) & ~size_t(255);
      }
      build_apply64(f.H, f.tr, f.cm, f.Xc, f.ldm, f.Ym, f.ldm, buf, tabs[p]);
    }
    tab_at[p] = blob.put(tabs[p].segs);
  }
  SLU_REQUIRE(blob.host.size() <= tab_bytes, "task table overflow");
  upload(h, blob, dtab);
  auto kern = group_step_kernel<double>;
  for (int p = 0; p < nphase; ++p)
    for (const sweep::LaunchPlan& lp : tabs[p].plan)
      if (lp.ctas > 0) ensure_smem(reinterpret_cast<const void*>(kern), lp.smem);
  stream_wait(st);   // tables in place before the capture
  cudaStream_t cs = nullptr;
  SLU_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  const long long n0 = launch_thread();
  try {
    SLU_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
      for (int p = 0; p < nphase; ++p) {
        const Phase& f = ph[p];
        if (f.kind >= 2) {
          if (f.ew.empty()) continue;
          long long nmax = 1;
          for (const EwSeg& e : f.ew) nmax = std::max(nmax, e.n);
          dim3 grid((unsigned)f.ew.size(),
                    (unsigned)std::min<long long>((nmax + 255) / 256, 64));
          ew_seg_k<<<grid, 256, 0, cs>>>(reinterpret_cast<const EwSeg*>(dtab + tab_at[p]));
          check_launch("ew_seg_k");
        } else if (!f.H.empty()) {
          launch_solve<double>(cs, tabs[p],
                               reinterpret_cast<const StepSeg<double>*>(dtab + tab_at[p]));
        }
      }
    } catch (...) {
      cudaStreamEndCapture(cs, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    SLU_CHECK_CUDA(cudaStreamEndCapture(cs, &g));
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
}

void hbs_apply_grouped(Handle& h, int count, Hbs* const* ops, const int* trans,
                       const double* const* X, const int* ldx, double* const* Y, const int* ldy,
                       const int* c) {
  SLU_REQUIRE(count >= 0 && (count == 0 || (ops && trans && X && ldx && Y && ldy && c)),
              "null argument");
  std::vector<const Hbs*> H;
  std::vector<int> tr, cm, lx, ly;
  std::vector<const double*> Xm;
  std::vector<double*> Ym;
  for (int i = 0; i < count; ++i) {
    SLU_REQUIRE(ops[i], "null operator");
    SLU_REQUIRE(c[i] >= 0, "bad right-hand-side count");
    if (c[i] == 0) continue;
    SLU_REQUIRE(X[i] && Y[i] && ldx[i] >= c[i] && ldy[i] >= c[i], "bad right-hand side");
    Hbs& Hi = *ops[i];
    SLU_REQUIRE(Hi.has_mats, "HBS factors not loaded");
    const int t = trans[i] ? 1 : 0;
    if (!Hi.has_apply[t]) {
      std::lock_guard<std::mutex> lock(Hi.lazy_mu);
      if (!Hi.has_apply[t]) hbs_make_apply(h, Hi, t == 1);
    }
    H.push_back(&Hi);
    tr.push_back(t);
    cm.push_back(c[i]);
    Xm.push_back(X[i]);
    lx.push_back(ldx[i]);
    Ym.push_back(Y[i]);
    ly.push_back(ldy[i]);
  }
  const int m = (int)H.size();
  if (m == 0) return;
  cudaStream_t st = h.stream;
  size_t nseg = 0;
  for (const Hbs* x : H) nseg += 2 * (size_t)x->L;
  Plan plan;
  plan.add(blob_bound(nseg * sizeof(StepSeg<double>), 1));
  for (int i = 0; i < m; ++i) plan.add(8 * hbs_apply_scratch_elems(*H[i], cm[i]));
  h.ws.reserve(plan.total(), st);
  char* dtab = h.ws.take<char>(plan.bytes[0]);
  std::vector<ApplyBufs<double>> buf(m);
  for (int i = 0; i < m; ++i)
    buf[i] = carve_apply(*H[i], cm[i], h.ws.take<double>(hbs_apply_scratch_elems(*H[i], cm[i])));
  StepTable<double> steps;
  build_apply64(H, tr, cm, Xm, lx, Ym, ly, buf, steps);
  Blob blob;
  const size_t at = blob.put(steps.segs);
  SLU_REQUIRE(blob.host.size() <= plan.bytes[0], "task table overflow");
  upload(h, blob, dtab);
  launch_solve<double>(st, steps, reinterpret_cast<const StepSeg<double>*>(dtab + at));
}

namespace {

// Inner sweep of the grouped refinement in T (dfloat or float).
inline void to_inner(cudaStream_t st, long long n, const double* x, dfloat* y) {
  to_dfs_k<<<gsz(n), 256, 0, st>>>(n, x, y);
  check_launch("to_dfs_k");
}
inline void to_inner(cudaStream_t st, long long n, const double* x, float* y) {
  to_f32_k<<<gsz(n), 256, 0, st>>>(n, x, y);
  check_launch("to_f32_k");
}
inline void accum_inner(cudaStream_t st, long long n, const dfloat* y, double* x, int init) {
  accum_dfs_k<<<gsz(n), 256, 0, st>>>(n, y, x, init);
  check_launch("accum_dfs_k");
}
inline void accum_inner(cudaStream_t st, long long n, const float* y, double* x, int init) {
  accum_k<<<gsz(n), 256, 0, st>>>(n, y, x, init);
  check_launch("accum_k");
}

// Buffers, task tables and launches of one grouped refinement: the members
// with columns, one contiguous device region (carved in the order below),
// and the launches of an iteration (cast, inner sweep, correction,
// double-float residual, column norms, norms to the host).
template <typename T>
struct GroupRefine {
  std::vector<int> idx, cm;
  std::vector<const Hbs*> H;
  int m = 0, C = 0;
  size_t E = 0, nseg = 0;
  std::vector<size_t> off, stride;
  Plan plan;
  double *dB = nullptr, *dX = nullptr, *dr = nullptr, *norms = nullptr;
  T* df = nullptr;
  dfloat *xdf = nullptr, *ydf = nullptr;
  StepTable<T> ssteps;
  StepTable<dfloat> dsteps;
  const StepSeg<T>* d_s = nullptr;
  const StepSeg<dfloat>* d_d = nullptr;
  const ColSeg* d_c = nullptr;
  const CopySeg *d_i = nullptr, *d_o = nullptr;
  dim3 cgrid;
  double* host = nullptr;   // pinned [bn | rn], C each

  // Members with columns, their factor copies, the region's sizes.
  bool init(Handle& h, int count, Hbs* const* ops, const double* const* B, const int* ldb,
            double* const* X, const int* ldx, const int* c) {
    constexpr bool kDf = sizeof(T) == 8;
    for (int i = 0; i < count; ++i) {
      SLU_REQUIRE(ops[i], "null operator");
      SLU_REQUIRE(c[i] >= 0, "bad right-hand-side count");
      if (c[i] == 0) continue;
      SLU_REQUIRE(B[i] && X[i] && ldb[i] >= c[i] && ldx[i] >= c[i], "bad right-hand side");
      SLU_REQUIRE(ops[i]->has_ulv, "ULV factors not computed");
      idx.push_back(i);
    }
    m = (int)idx.size();
    if (m == 0) return false;
    for (int i : idx) {
      if (kDf && !ops[i]->has_dfs) hbs_make_dfs(h, *ops[i]);
      if (!kDf && !ops[i]->has_f32) hbs_make_f32(h, *ops[i]);
      if (!ops[i]->has_df) hbs_make_df(h, *ops[i]);
    }
    H.resize(m);
    cm.resize(m);
    off.resize(m);
    stride.resize(m);
    for (int j = 0; j < m; ++j) {
      H[j] = ops[idx[j]];
      cm[j] = c[idx[j]];
      off[j] = E;
      E += (size_t)H[j]->N * cm[j];
      C += cm[j];
      stride[j] = round64((size_t)H[j]->N * cm[j]);
      nseg += 2 * (size_t)H[j]->L;
    }
    plan.add(blob_bound(nseg * (sizeof(StepSeg<T>) + sizeof(StepSeg<dfloat>)) +
                            (size_t)C * sizeof(ColSeg) + 2 * m * sizeof(CopySeg),
                        5));
    plan.add(8 * E);  // B
    plan.add(8 * E);  // X
    plan.add(8 * E);  // r
    plan.add(sizeof(T) * E);  // inner right-hand sides / corrections
    plan.add(16 * (size_t)C);  // [bn | rn]
    plan.add(sizeof(dfloat) * E);  // X as double-float pairs (residual apply input)
    plan.add(sizeof(dfloat) * E);  // A X as double-float pairs
    for (int j = 0; j < m; ++j) plan.add(5 * stride[j] * sizeof(T));
    for (int j = 0; j < m; ++j)
      plan.add(sizeof(dfloat) * hbs_apply_scratch_elems(*H[j], cm[j]));
    return true;
  }

  // Carves the region (plan.total() bytes at base), builds the task tables
  // and uploads them on h's stream.
  void carve(Handle& h, char* base, const double* const* B, const int* ldb, double* const* X,
             const int* ldx) {
    size_t at = 0;
    auto take = [&](size_t bytes) {
      char* p = base + at;
      at += (bytes + 255) & ~size_t(255);
      return p;
    };
    char* dtab = take(plan.bytes[0]);
    dB = reinterpret_cast<double*>(take(8 * E));
    dX = reinterpret_cast<double*>(take(8 * E));
    dr = reinterpret_cast<double*>(take(8 * E));
    df = reinterpret_cast<T*>(take(sizeof(T) * E));
    norms = reinterpret_cast<double*>(take(16 * (size_t)C));
    xdf = reinterpret_cast<dfloat*>(take(sizeof(dfloat) * E));
    ydf = reinterpret_cast<dfloat*>(take(sizeof(dfloat) * E));
    std::vector<SolveBufs<T>> sbuf(m);
    for (int j = 0; j < m; ++j) {
      T* s = reinterpret_cast<T*>(take(5 * stride[j] * sizeof(T)));
      sbuf[j].ru = s;
      for (int q = 0; q < 4; ++q) sbuf[j].P[q] = s + (q + 1) * stride[j];
    }
    std::vector<ApplyBufs<dfloat>> abuf(m);
    for (int j = 0; j < m; ++j)
      abuf[j] = carve_apply(*H[j], cm[j],
                            reinterpret_cast<dfloat*>(take(sizeof(dfloat) *
                                                           hbs_apply_scratch_elems(*H[j], cm[j]))));
    std::vector<T*> fB(m);
    std::vector<const dfloat*> xX(m);
    std::vector<dfloat*> rY(m);
    for (int j = 0; j < m; ++j) {
      fB[j] = df + off[j];
      xX[j] = xdf + off[j];
      rY[j] = ydf + off[j];
    }
    build_solve<T>(H, cm, fB, cm, sbuf, ssteps);
    build_apply_df(H, cm, xX, rY, abuf, dsteps);
    std::vector<ColSeg> cols;
    cols.reserve(C);
    std::vector<CopySeg> cin(m), cpy_out(m);
    long long maxe = 1;
    for (int j = 0; j < m; ++j) {
      for (int q = 0; q < cm[j]; ++q) cols.push_back({(long long)(off[j] + q), H[j]->N, cm[j]});
      cin[j] = {B[idx[j]], dB + off[j], ldb[idx[j]], cm[j], H[j]->N, cm[j]};
      cpy_out[j] = {dX + off[j], X[idx[j]], cm[j], ldx[idx[j]], H[j]->N, cm[j]};
      maxe = std::max(maxe, (long long)H[j]->N * cm[j]);
    }
    Blob blob;
    const size_t a_s = blob.put(ssteps.segs), a_d = blob.put(dsteps.segs), a_c = blob.put(cols),
                 a_i = blob.put(cin), a_o = blob.put(cpy_out);
    SLU_REQUIRE(blob.host.size() <= plan.bytes[0], "task table overflow");
    upload(h, blob, dtab);
    d_s = reinterpret_cast<const StepSeg<T>*>(dtab + a_s);
    d_d = reinterpret_cast<const StepSeg<dfloat>*>(dtab + a_d);
    d_c = reinterpret_cast<const ColSeg*>(dtab + a_c);
    d_i = reinterpret_cast<const CopySeg*>(dtab + a_i);
    d_o = reinterpret_cast<const CopySeg*>(dtab + a_o);
    cgrid = dim3(m, (unsigned)std::min<long long>(64, (maxe + 1023) / 1024));
  }

  // Shared-memory limits of every step launch (before a stream capture).
  void prepare_launches() const {
    for (const sweep::LaunchPlan& p : ssteps.plan)
      if (p.ctas > 0) ensure_smem(reinterpret_cast<const void*>(group_step_kernel<T>), p.smem);
    for (const sweep::LaunchPlan& p : dsteps.plan)
      if (p.ctas > 0)
        ensure_smem(reinterpret_cast<const void*>(group_step_kernel<dfloat>), p.smem);
  }

  void copy_in(cudaStream_t st) const {
    seg_copy_k<<<cgrid, 256, 0, st>>>(d_i);
    check_launch("seg_copy_k");
  }
  void copy_out(cudaStream_t st) const {
    seg_copy_k<<<cgrid, 256, 0, st>>>(d_o);
    check_launch("seg_copy_k");
  }

  void iteration(cudaStream_t st, bool first) const {
    const long long En = (long long)E;
    if (first) {
      colnorm_seg_k<<<C, 256, 0, st>>>(d_c, dB, norms);
      check_launch("colnorm_seg_k");
      SLU_CHECK_CUDA(cudaMemcpyAsync(host, norms, 8 * (size_t)C, cudaMemcpyDeviceToHost, st));
    }
    to_inner(st, En, first ? dB : dr, df);
    launch_solve<T>(st, ssteps, d_s);
    accum_inner(st, En, df, dX, first ? 1 : 0);
    to_dfs_k<<<gsz(En), 256, 0, st>>>(En, dX, xdf);
    check_launch("to_dfs_k");
    launch_solve<dfloat>(st, dsteps, d_d);
    resid_dfs_k<<<gsz(En), 256, 0, st>>>(En, dB, ydf, dr);
    check_launch("resid_dfs_k");
    colnorm_seg_k<<<C, 256, 0, st>>>(d_c, dr, norms + C);
    check_launch("colnorm_seg_k");
    SLU_CHECK_CUDA(
        cudaMemcpyAsync(host + C, norms + C, 8 * (size_t)C, cudaMemcpyDeviceToHost, st));
  }

  // Worst relative residual over all columns (host norms of the last
  // iteration); member[j] = member j's worst.
  double check(std::vector<double>& member) const {
    double worst = 0.0;
    int col = 0;
    member.assign(m, 0.0);
    for (int j = 0; j < m; ++j) {
      double w = 0.0;
      for (int q = 0; q < cm[j]; ++q, ++col) {
        const double bj = host[col], rj = host[C + col];
        w = std::max(w, std::sqrt(rj) / (bj > 0 ? std::sqrt(bj) : 1.0));
      }
      member[j] = w;
      worst = std::max(worst, w);
    }
    return worst;
  }
};

// The refinement loop: first() then next() until every column reaches tol
// (float32 inner sweeps: no check before the second correction).
template <typename T, class First, class Next>
double refine_loop(cudaStream_t st, const GroupRefine<T>& g, double tol, int maxit, First first,
                   Next next, int* iters, std::vector<double>& member) {
  constexpr bool kDf = sizeof(T) == 8;
  first();
  int it = 1;
  double worst = 0.0;
  for (;;) {
    if (!kDf && it < 2 && it < maxit && tol < 1e-6) {
      next();
      ++it;
      continue;
    }
    stream_wait(st);
    worst = g.check(member);
    if (worst <= tol || it >= maxit) break;
    next();
    ++it;
  }
  if (iters) *iters = it;
  return worst;
}

template <typename T>
void refine_grouped(Handle& h, int count, Hbs* const* ops, const double* const* B,
                    const int* ldb, double* const* X, const int* ldx, const int* c, double tol,
                    int maxit, int* iters, double* relres) {
  if (relres)
    for (int i = 0; i < count; ++i) relres[i] = 0.0;
  if (iters) *iters = 0;
  GroupRefine<T> g;
  if (!g.init(h, count, ops, B, ldb, X, ldx, c)) return;
  cudaStream_t st = h.stream;
  h.ws.reserve(g.plan.total(), st);
  g.carve(h, h.ws.take<char>(g.plan.total()), B, ldb, X, ldx);
  g.host = reinterpret_cast<double*>(h.readback.acquire(16 * (size_t)g.C));
  std::vector<double> member;
  const double worst = refine_loop(
      st, g, tol, maxit,
      [&] {
        g.copy_in(st);
        g.iteration(st, true);
      },
      [&] { g.iteration(st, false); }, iters, member);
  h.readback.release(st);
  g.copy_out(st);
  if (relres)
    for (int j = 0; j < g.m; ++j) relres[g.idx[j]] = member[j];
  if (worst > tol) throw Error(SLU_ERR_NOT_CONVERGED, "refinement did not reach the tolerance");
}

// A grouped refinement for fixed blocks: the region, task tables and pinned
// norms owned by the plan; one iteration captured as CUDA graphs (the first
// with the copy-in and the norms of B, the next ones, the copy-out).
template <typename T>
struct GroupRefinePlanT : GroupRefinePlan {
  GroupRefine<T> g;
  DevBuf region;
  double* pinned = nullptr;
  cudaGraphExec_t first = nullptr, next = nullptr, out = nullptr;
  long long kf = 0, kn = 0, ko = 0;
  ~GroupRefinePlanT() override {
    if (first) cudaGraphExecDestroy(first);
    if (next) cudaGraphExecDestroy(next);
    if (out) cudaGraphExecDestroy(out);
    if (pinned) cudaFreeHost(pinned);
  }

  template <class F>
  cudaGraphExec_t capture(cudaStream_t cs, F enqueue, long long& kernels) {
    cudaGraph_t gr = nullptr;
    const long long n0 = launch_thread();
    SLU_CHECK_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue();
    } catch (...) {
      cudaStreamEndCapture(cs, &gr);
      if (gr) cudaGraphDestroy(gr);
      throw;
    }
    SLU_CHECK_CUDA(cudaStreamEndCapture(cs, &gr));
    kernels = launch_thread() - n0;
    launch_total() -= kernels;
    launch_thread() = n0;
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ex, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess)
      throw Error(SLU_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return ex;
  }

  void create(Handle& h, int count, Hbs* const* ops, const double* const* B, const int* ldb,
              double* const* X, const int* ldx, const int* c) {
    total = count;
    if (!g.init(h, count, ops, B, ldb, X, ldx, c)) return;
    for (const Hbs* x : g.H) {
      alive.push_back(x->alive);
      gen.push_back(x->sweep_gen);
      H.push_back(x);
    }
    idx = g.idx;
    cudaStream_t st = h.stream;
    region.alloc(g.plan.total(), st);
    g.carve(h, static_cast<char*>(region.p), B, ldb, X, ldx);
    SLU_CHECK_CUDA(cudaMallocHost(&pinned, 16 * (size_t)g.C));
    g.host = pinned;
    g.prepare_launches();
    stream_wait(st);   // region and tables in place
    cudaStream_t cs = nullptr;
    SLU_CHECK_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    try {
      first = capture(cs, [&] {
        g.copy_in(cs);
        g.iteration(cs, true);
      }, kf);
      next = capture(cs, [&] { g.iteration(cs, false); }, kn);
      out = capture(cs, [&] { g.copy_out(cs); }, ko);
    } catch (...) {
      cudaStreamDestroy(cs);
      throw;
    }
    SLU_CHECK_CUDA(cudaStreamDestroy(cs));
  }

  void run(Handle& h, double tol, int maxit, int* iters, double* relres) override {
    SLU_REQUIRE(maxit >= 1, "bad iteration limit");
    for (size_t i = 0; i < H.size(); ++i) {
      if (alive[i].expired())
        throw Error(SLU_ERR_STATE, "an operator of the refinement plan was destroyed");
      if (H[i]->sweep_gen != gen[i])
        throw Error(SLU_ERR_STATE, "an operator was refactored after the plan was made");
    }
    if (relres)
      for (int i = 0; i < total; ++i) relres[i] = 0.0;
    if (iters) *iters = 0;
    if (!first) return;
    cudaStream_t st = h.stream;
    std::vector<double> member;
    const double worst = refine_loop(
        st, g, tol, maxit,
        [&] {
          SLU_CHECK_CUDA(cudaGraphLaunch(first, st));
          count_launches(kf);
        },
        [&] {
          SLU_CHECK_CUDA(cudaGraphLaunch(next, st));
          count_launches(kn);
        },
        iters, member);
    SLU_CHECK_CUDA(cudaGraphLaunch(out, st));
    count_launches(ko);
    if (relres)
      for (int j = 0; j < g.m; ++j) relres[idx[j]] = member[j];
    if (worst > tol) throw Error(SLU_ERR_NOT_CONVERGED, "refinement did not reach the tolerance");
  }
};

}  // namespace

void hbs_refine_grouped(Handle& h, int count, Hbs* const* ops, const double* const* B,
                        const int* ldb, double* const* X, const int* ldx, const int* c,
                        double tol, int maxit, int* iters, double* relres) {
  SLU_REQUIRE(count >= 0 && (count == 0 || (ops && B && ldb && X && ldx && c)),
              "null argument");
  SLU_REQUIRE(maxit >= 1, "bad iteration limit");
  // double-float inner sweeps unless every member asks for float32
  bool f32 = count > 0;
  for (int i = 0; i < count; ++i) f32 = f32 && ops[i] && ops[i]->refine_inner == 0;
  if (f32) refine_grouped<float>(h, count, ops, B, ldb, X, ldx, c, tol, maxit, iters, relres);
  else refine_grouped<dfloat>(h, count, ops, B, ldb, X, ldx, c, tol, maxit, iters, relres);
}

std::unique_ptr<GroupRefinePlan> grouped_refine_plan_create(Handle& h, int count,
                                                            Hbs* const* ops, const double* const* B,
                                                            const int* ldb, double* const* X,
                                                            const int* ldx, const int* c) {
  SLU_REQUIRE(count >= 0 && (count == 0 || (ops && B && ldb && X && ldx && c)),
              "null argument");
  bool f32 = count > 0;
  for (int i = 0; i < count; ++i) f32 = f32 && ops[i] && ops[i]->refine_inner == 0;
  if (f32) {
    auto p = std::make_unique<GroupRefinePlanT<float>>();
    p->create(h, count, ops, B, ldb, X, ldx, c);
    return p;
  }
  auto p = std::make_unique<GroupRefinePlanT<dfloat>>();
  p->create(h, count, ops, B, ldb, X, ldx, c);
  return p;
}

}  // namespace slu
