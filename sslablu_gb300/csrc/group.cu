// Grouped HBS solves: many operators of uneven sizes, one launch per tree step.
//
// The reference solves one operator per call (HBSnew.HBSMAT.solve,
// matAssembly/HBS/HBSnew.py:393-416, through ULVsparse.solve,
// matAssembly/HBS/ULVsparse.py:296-327); the slab solvers call it for every
// block of every level.  Solving a group of operators with the per-operator
// kernels costs 2L-1 launches per operator, each too small to fill 152 SMs.
// Here each tree step of every member becomes a *segment* of one launch: a
// task table lists, per segment, the member's factors, buffers and column
// chunking, and the CTA range it owns; a CTA finds its segment by binary
// search over the range starts and runs the same device body as the
// per-operator kernel (ulv_bodies.cuh, df_bodies.cuh).  The schedule is
//   forward  t = 0 .. maxL-2   (members with L_i >= t + 2)
//   root                         (every member)
//   backward t = maxL-2 .. 0   (members with L_i >= t + 2)
// so members of different depths share launches, and each member's own
// sequence of steps (and of ping-pong buffers) is exactly its solo sequence.
//
// Mixed-precision refinement of a group (hbs_refine_grouped) runs the same
// loop as refine.cu over concatenated buffers: one launch per elementwise step
// for the whole group, the float32 grouped sweep, the grouped double-float
// apply, and segmented column norms.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "df_bodies.cuh"
#include "hbs.cuh"
#include "refine_kernels.cuh"
#include "ulv_bodies.cuh"

namespace slu {
namespace {

constexpr int kThreads = 256;
constexpr size_t kSmemLimit = 200 * 1024;

using dfk::DF;

// One tree step of one member in a grouped ULV sweep.
template <typename T>
struct SolveSeg {
  int kind;  // 0 forward, 1 root, 2 backward
  int n, nu, k, c, cpb, nchunk, cta0, lds, ldb;
  const T *Q, *R, *W, *U, *D, *Uu;
  const T* src;
  const int64_t* perm;
  T *ru, *dst, *Yin, *Vin, *Yout, *Vout, *B;
};

// One tree step of one member in a grouped double-float apply.
struct DfSeg {
  int kind;  // 0 upward, 1 root or downward
  int n, k, c, cpb, nchunk, cta0, ldx, ldy;
  const float *Fh, *Fl, *Dh, *Dl;  // upward: V; downward: U (Fh/Fl) and D
  const DF *in, *uin, *vv;
  const double* X;
  const int64_t* perm;
  DF* out;
  double* Y;
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
__global__ void __launch_bounds__(kThreads)
group_solve_kernel(const SolveSeg<T>* __restrict__ segs, int nseg) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const SolveSeg<T>& s = segs[find_seg(segs, nseg)];
  const int local = blockIdx.x - s.cta0;
  const int b = local / s.nchunk;
  const int c0 = (local - b * s.nchunk) * s.cpb;
  const int nc = min(s.cpb, s.c - c0);
  if (nc <= 0) return;
  if (s.kind == 0)
    ulvk::ulv_fwd_body<T>(sm_raw, b, c0, nc, s.n, s.nu, s.k, s.Q, s.src, s.lds, s.perm, s.ru,
                          s.dst, s.c, s.cpb);
  else if (s.kind == 1)
    ulvk::ulv_root_body<T, false>(sm_raw, c0, nc, s.n, s.Q, s.R, s.D, s.src, s.lds, s.perm, s.Yout,
                           s.Vout, s.B, s.ldb, s.c, s.cpb);
  else
    ulvk::ulv_bwd_body<T, false>(sm_raw, b, c0, nc, s.n, s.nu, s.k, s.ru, s.Uu, s.R, s.W, s.U, s.D,
                          s.Vin, s.Yin, s.Yout, s.Vout, s.perm, s.B, s.ldb, s.c, s.cpb);
}

__global__ void __launch_bounds__(kThreads)
group_df_kernel(const DfSeg* __restrict__ segs, int nseg) {
  extern __shared__ __align__(16) float smf[];
  const DfSeg& s = segs[find_seg(segs, nseg)];
  const int local = blockIdx.x - s.cta0;
  const int b = local / s.nchunk;
  const int c0 = (local - b * s.nchunk) * s.cpb;
  const int nc = min(s.cpb, s.c - c0);
  if (nc <= 0) return;
  if (s.kind == 0)
    dfk::df_up_body(smf, b, c0, nc, s.n, s.k, s.Fh, s.Fl, s.X, s.ldx, s.perm, s.in, s.out, s.c,
                    s.cpb);
  else
    dfk::df_down_body(smf, b, c0, nc, s.n, s.k, s.Fh, s.Fl, s.Dh, s.Dl, s.uin, s.vv, s.X, s.ldx,
                      s.perm, s.out, s.Y, s.ldy, s.c, s.cpb);
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

// ------------------------------------------------------------------ host side
struct Geom {
  int Nb, c;
  size_t a, b;  // shared memory bytes of a CTA = a + b * cpb
};

// Step tables: segments of every step, back to back.
template <class S>
struct Steps {
  std::vector<S> segs;
  std::vector<int> off, ctas;
  std::vector<size_t> smem;
  std::vector<Geom> g;  // geometry of the step being built
  void begin() {
    off.push_back((int)segs.size());
    g.clear();
  }
  // Column chunks for the step just built: the widest chunk m (at most
  // mstart) that still gives `target` CTAs, halving down to mmin; each
  // segment then narrows its own chunk until its CTA fits in shared memory.
  void end(int mstart, int mmin, long long target) {
    auto count = [&](int m) {
      long long t = 0;
      for (const Geom& x : g) {
        const int cp = std::min(x.c, m);
        t += (long long)x.Nb * ((x.c + cp - 1) / cp);
      }
      return t;
    };
    int m = std::max(mstart, 1);
    while (m > mmin && count(m) < target) m = (m + 1) / 2;
    long long cta = 0;
    size_t sm = 0;
    const size_t first = off.back();
    for (size_t i = 0; i < g.size(); ++i) {
      S& s = segs[first + i];
      int cpb = std::min(g[i].c, m);
      while (cpb > 1 && g[i].a + g[i].b * cpb > kSmemLimit) cpb = (cpb + 1) / 2;
      SLU_REQUIRE(g[i].a + g[i].b * cpb <= kSmemLimit, "block too large for the grouped solve");
      s.cpb = cpb;
      s.nchunk = (g[i].c + cpb - 1) / cpb;
      s.cta0 = (int)cta;
      cta += (long long)g[i].Nb * s.nchunk;
      sm = std::max(sm, g[i].a + g[i].b * cpb);
    }
    SLU_REQUIRE(cta < (1LL << 31), "grouped step too large");
    ctas.push_back((int)cta);
    smem.push_back(sm);
  }
  int nsteps() const { return (int)ctas.size(); }
  int count(int s) const {
    return (s + 1 < (int)off.size() ? off[s + 1] : (int)segs.size()) - off[s];
  }
};

// Per-member device buffers of a grouped ULV sweep (five of `stride`).
template <typename T>
struct SolveBufs {
  T* ru;
  T* P[4];
};

// Builds the step tables of a grouped mode-N ULV sweep; B[i] is solved in place.
template <typename T>
void build_solve(const std::vector<const Hbs*>& H, const std::vector<int>& c,
                 const std::vector<T*>& B, const std::vector<int>& ldb,
                 const std::vector<SolveBufs<T>>& buf, Steps<SolveSeg<T>>& st) {
  using F = FacPtr<T>;
  const int m = (int)H.size();
  int maxL = 0, maxc = 1;
  for (int i = 0; i < m; ++i) {
    maxL = std::max(maxL, H[i]->L);
    maxc = std::max(maxc, c[i]);
  }
  const bool f64 = sizeof(T) == 8;
  const long long target = (f64 ? 2 : 1) * (long long)num_sms();
  const int mstart = f64 ? maxc : std::min(maxc, 16), mmin = f64 ? 1 : 4;
  const size_t e = sizeof(T);
  for (int t = 0; t + 1 < maxL; ++t) {
    st.begin();
    for (int i = 0; i < m; ++i) {
      if (H[i]->L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      SolveSeg<T> s{};
      s.kind = 0;
      s.n = l.n; s.nu = l.nu; s.k = l.k; s.c = c[i];
      s.Q = F::Q(l);
      s.src = t == 0 ? B[i] : buf[i].P[(t - 1) & 1];
      s.lds = t == 0 ? ldb[i] : c[i];
      s.perm = t == 0 ? H[i]->perm.as<int64_t>() : nullptr;
      s.ru = buf[i].ru + H[i]->NN[t] * c[i];
      s.dst = buf[i].P[t & 1];
      st.segs.push_back(s);
      st.g.push_back({l.Nb, c[i], e * ulvk::ulv_fwd_smem(l.n, 0), e * 2 * l.n});
    }
    st.end(mstart, mmin, target);
  }
  st.begin();
  for (int i = 0; i < m; ++i) {
    const int L = H[i]->L;
    const Level& r = H[i]->lv[L - 1];
    SolveSeg<T> s{};
    s.kind = 1;
    s.n = r.n; s.c = c[i];
    s.Q = F::Q(r); s.R = F::R(r); s.D = F::D(r);
    s.src = L == 1 ? B[i] : buf[i].P[(L - 2) & 1];
    s.lds = L == 1 ? ldb[i] : c[i];
    s.perm = L == 1 ? H[i]->perm.as<int64_t>() : nullptr;
    s.Yout = buf[i].P[2];
    s.Vout = buf[i].P[3];
    s.B = B[i];
    s.ldb = ldb[i];
    st.segs.push_back(s);
    st.g.push_back({1, c[i], e * ulvk::ulv_root_smem(r.n, 0, false), e * 2 * r.n});
  }
  st.end(mstart, mmin, target);
  for (int t = maxL - 2; t >= 0; --t) {
    st.begin();
    for (int i = 0; i < m; ++i) {
      const int L = H[i]->L;
      if (L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      const int in = ((L - 2 - t) % 2 == 0) ? 2 : 0, out = in == 2 ? 0 : 2;
      SolveSeg<T> s{};
      s.kind = 2;
      s.n = l.n; s.nu = l.nu; s.k = l.k; s.c = c[i];
      s.ru = buf[i].ru + H[i]->NN[t] * c[i];
      s.Uu = F::Uu(l); s.R = F::R(l); s.W = F::W(l); s.U = F::U(l); s.D = F::D(l);
      s.Vin = buf[i].P[in + 1];
      s.Yin = buf[i].P[in];
      s.Yout = buf[i].P[out];
      s.Vout = buf[i].P[out + 1];
      s.perm = t == 0 ? H[i]->perm.as<int64_t>() : nullptr;
      s.B = B[i];
      s.ldb = ldb[i];
      st.segs.push_back(s);
      st.g.push_back({l.Nb, c[i], e * ulvk::ulv_bwd_smem(l.n, l.nu, l.k, 0, false, t == 0),
                      e * (2 * l.k + l.nu + 2 * l.n)});
    }
    st.end(mstart, mmin, target);
  }
}

// Per-member device buffers of a grouped double-float apply.
struct DfBufs {
  std::vector<DF*> VV;  // VV[t] for t >= 1
  DF* u[2];
};

DfBufs carve_df(const Hbs& H, int c, void* scratch) {
  DfBufs d;
  DF* base = reinterpret_cast<DF*>(scratch);
  d.VV.assign(H.L, nullptr);
  size_t off = 0;
  for (int t = 0; t + 1 < H.L; ++t) {
    d.VV[t + 1] = base + off;
    off += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 31) & ~size_t(31);
  }
  d.u[0] = base + off;
  d.u[1] = base + off + (((size_t)H.N * c + 31) & ~size_t(31));
  return d;
}

// Step tables of a grouped double-float apply Y[i] = A_i X[i] (the recursion
// of hbs_apply_df.cu).
void build_df(const std::vector<const Hbs*>& H, const std::vector<int>& c,
              const std::vector<const double*>& X, const std::vector<int>& ldx,
              const std::vector<double*>& Y, const std::vector<int>& ldy,
              const std::vector<DfBufs>& buf, Steps<DfSeg>& st) {
  const int m = (int)H.size();
  int maxL = 0, maxc = 1;
  for (int i = 0; i < m; ++i) {
    maxL = std::max(maxL, H[i]->L);
    maxc = std::max(maxc, c[i]);
  }
  const long long target = num_sms();
  const int mstart = std::min(maxc, 16), mmin = 2;
  for (int t = 0; t + 1 < maxL; ++t) {
    st.begin();
    for (int i = 0; i < m; ++i) {
      if (H[i]->L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      DfSeg s{};
      s.kind = 0;
      s.n = l.n; s.k = l.k; s.c = c[i];
      s.Fh = l.Vh.as<float>(); s.Fl = l.Vl.as<float>();
      s.X = t == 0 ? X[i] : nullptr;
      s.ldx = ldx[i];
      s.perm = t == 0 ? H[i]->perm.as<int64_t>() : nullptr;
      s.in = buf[i].VV[t];
      s.out = buf[i].VV[t + 1];
      st.segs.push_back(s);
      st.g.push_back({l.Nb, c[i], 4 * 2 * (size_t)l.n * (l.k + 1), 4 * 2 * (size_t)l.n});
    }
    st.end(mstart, mmin, target);
  }
  st.begin();
  for (int i = 0; i < m; ++i) {
    const int L = H[i]->L;
    const Level& r = H[i]->lv[L - 1];
    DfSeg s{};
    s.kind = 1;
    s.n = r.n; s.k = 0; s.c = c[i];
    s.Dh = r.Dh.as<float>(); s.Dl = r.Dl.as<float>();
    if (L == 1) {
      s.X = X[i];
      s.ldx = ldx[i];
      s.perm = H[i]->perm.as<int64_t>();
      s.Y = Y[i];
      s.ldy = ldy[i];
    } else {
      s.vv = buf[i].VV[L - 1];
      s.out = buf[i].u[0];
    }
    st.segs.push_back(s);
    st.g.push_back({1, c[i], 4 * 2 * (size_t)r.n * (r.n + 1), 4 * 4 * (size_t)r.n});
  }
  st.end(mstart, mmin, target);
  for (int t = maxL - 2; t >= 0; --t) {
    st.begin();
    for (int i = 0; i < m; ++i) {
      const int L = H[i]->L;
      if (L < t + 2) continue;
      const Level& l = H[i]->lv[t];
      const int cur = (L - 2 - t) & 1;
      const bool leaf = t == 0;
      DfSeg s{};
      s.kind = 1;
      s.n = l.n; s.k = l.k; s.c = c[i];
      s.Fh = l.Uh.as<float>(); s.Fl = l.Ul.as<float>();
      s.Dh = l.Dh.as<float>(); s.Dl = l.Dl.as<float>();
      s.uin = buf[i].u[cur];
      s.vv = leaf ? nullptr : buf[i].VV[t];
      s.X = leaf ? X[i] : nullptr;
      s.ldx = ldx[i];
      s.perm = leaf ? H[i]->perm.as<int64_t>() : nullptr;
      s.out = leaf ? nullptr : buf[i].u[cur ^ 1];
      s.Y = leaf ? Y[i] : nullptr;
      s.ldy = ldy[i];
      st.segs.push_back(s);
      st.g.push_back({l.Nb, c[i], 4 * 2 * (size_t)l.n * (l.n + 1),
                      4 * (4 * (size_t)l.n + 2 * (size_t)l.k)});
    }
    st.end(mstart, mmin, target);
  }
}

template <typename K>
void set_smem(K kern, size_t bytes) {
  ensure_smem(reinterpret_cast<const void*>(kern), bytes);
}

template <typename T>
void launch_solve(cudaStream_t st, const Steps<SolveSeg<T>>& s, const SolveSeg<T>* dsegs) {
  auto kern = group_solve_kernel<T>;
  for (int i = 0; i < s.nsteps(); ++i) {
    if (s.ctas[i] == 0) continue;
    set_smem(kern, s.smem[i]);
    kern<<<s.ctas[i], kThreads, s.smem[i], st>>>(dsegs + s.off[i], s.count(i));
    check_launch("group_solve_kernel");
  }
}

void launch_df(cudaStream_t st, const Steps<DfSeg>& s, const DfSeg* dsegs) {
  auto kern = group_df_kernel;
  for (int i = 0; i < s.nsteps(); ++i) {
    if (s.ctas[i] == 0) continue;
    set_smem(kern, s.smem[i]);
    kern<<<s.ctas[i], kThreads, s.smem[i], st>>>(dsegs + s.off[i], s.count(i));
    check_launch("group_df_kernel");
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
  plan.add(blob_bound(nseg * sizeof(SolveSeg<double>), 1));
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
  Steps<SolveSeg<double>> steps;
  build_solve<double>(H, cm, Bm, ldm, buf, steps);
  Blob blob;
  const size_t at = blob.put(steps.segs);
  SLU_REQUIRE(blob.host.size() <= plan.bytes[0], "task table overflow");
  upload(h, blob, dtab);
  launch_solve<double>(st, steps, reinterpret_cast<const SolveSeg<double>*>(dtab + at));
}

void hbs_refine_grouped(Handle& h, int count, Hbs* const* ops, const double* const* B,
                        const int* ldb, double* const* X, const int* ldx, const int* c,
                        double tol, int maxit, int* iters, double* relres) {
  SLU_REQUIRE(count >= 0 && (count == 0 || (ops && B && ldb && X && ldx && c)),
              "null argument");
  SLU_REQUIRE(maxit >= 1, "bad iteration limit");
  std::vector<int> idx;
  for (int i = 0; i < count; ++i) {
    SLU_REQUIRE(ops[i], "null operator");
    SLU_REQUIRE(c[i] >= 0, "bad right-hand-side count");
    if (relres) relres[i] = 0.0;
    if (c[i] == 0) continue;
    SLU_REQUIRE(B[i] && X[i] && ldb[i] >= c[i] && ldx[i] >= c[i], "bad right-hand side");
    SLU_REQUIRE(ops[i]->has_ulv, "ULV factors not computed");
    idx.push_back(i);
  }
  if (iters) *iters = 0;
  const int m = (int)idx.size();
  if (m == 0) return;
  cudaStream_t st = h.stream;
  for (int i : idx) {
    if (!ops[i]->has_f32) hbs_make_f32(h, *ops[i]);
    if (!ops[i]->has_df) hbs_make_df(h, *ops[i]);
  }
  std::vector<const Hbs*> H(m);
  std::vector<int> cm(m);
  std::vector<size_t> off(m), stride(m);
  size_t E = 0;
  int C = 0;
  size_t nseg = 0;
  for (int j = 0; j < m; ++j) {
    H[j] = ops[idx[j]];
    cm[j] = c[idx[j]];
    off[j] = E;
    E += (size_t)H[j]->N * cm[j];
    C += cm[j];
    stride[j] = round64((size_t)H[j]->N * cm[j]);
    nseg += 2 * (size_t)H[j]->L;
  }
  // device regions
  Plan plan;
  const size_t tab_bytes = blob_bound(nseg * (sizeof(SolveSeg<float>) + sizeof(DfSeg)) +
                                          (size_t)C * sizeof(ColSeg) + 2 * m * sizeof(CopySeg),
                                      5);
  plan.add(tab_bytes);
  plan.add(8 * E);  // B
  plan.add(8 * E);  // X
  plan.add(8 * E);  // r
  plan.add(4 * E);  // f
  plan.add(16 * (size_t)C);  // [bn | rn]
  for (int j = 0; j < m; ++j) plan.add(5 * stride[j] * sizeof(float));
  for (int j = 0; j < m; ++j) plan.add(hbs_apply_df_scratch_bytes(*H[j], cm[j]));
  h.ws.reserve(plan.total(), st);
  char* dtab = h.ws.take<char>(plan.bytes[0]);
  double* dB = h.ws.take<double>(E);
  double* dX = h.ws.take<double>(E);
  double* dr = h.ws.take<double>(E);
  float* df = h.ws.take<float>(E);
  double* norms = h.ws.take<double>(2 * (size_t)C);
  std::vector<SolveBufs<float>> sbuf(m);
  for (int j = 0; j < m; ++j) {
    float* s = h.ws.take<float>(5 * stride[j]);
    sbuf[j].ru = s;
    for (int q = 0; q < 4; ++q) sbuf[j].P[q] = s + (q + 1) * stride[j];
  }
  std::vector<DfBufs> dbuf(m);
  for (int j = 0; j < m; ++j)
    dbuf[j] = carve_df(*H[j], cm[j], h.ws.take<char>(plan.bytes[6 + m + j]));
  // task tables
  std::vector<float*> fB(m);
  std::vector<const double*> xX(m);
  std::vector<double*> rY(m);
  for (int j = 0; j < m; ++j) {
    fB[j] = df + off[j];
    xX[j] = dX + off[j];
    rY[j] = dr + off[j];
  }
  Steps<SolveSeg<float>> ssteps;
  build_solve<float>(H, cm, fB, cm, sbuf, ssteps);
  Steps<DfSeg> dsteps;
  build_df(H, cm, xX, cm, rY, cm, dbuf, dsteps);
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
  SLU_REQUIRE(blob.host.size() <= tab_bytes, "task table overflow");
  upload(h, blob, dtab);
  const auto* d_s = reinterpret_cast<const SolveSeg<float>*>(dtab + a_s);
  const auto* d_d = reinterpret_cast<const DfSeg*>(dtab + a_d);
  const auto* d_c = reinterpret_cast<const ColSeg*>(dtab + a_c);
  const auto* d_i = reinterpret_cast<const CopySeg*>(dtab + a_i);
  const auto* d_o = reinterpret_cast<const CopySeg*>(dtab + a_o);
  const dim3 cgrid(m, (unsigned)std::min<long long>(64, (maxe + 1023) / 1024));
  const long long En = (long long)E;
  double* host = reinterpret_cast<double*>(h.readback.acquire(16 * (size_t)C));

  auto iteration = [&](bool first) {
    if (first) {
      colnorm_seg_k<<<C, 256, 0, st>>>(d_c, dB, norms);
      check_launch("colnorm_seg_k");
      SLU_CHECK_CUDA(
          cudaMemcpyAsync(host, norms, 8 * (size_t)C, cudaMemcpyDeviceToHost, st));
    }
    to_f32_k<<<gsz(En), 256, 0, st>>>(En, first ? dB : dr, df);
    check_launch("to_f32_k");
    launch_solve<float>(st, ssteps, d_s);
    accum_k<<<gsz(En), 256, 0, st>>>(En, df, dX, first ? 1 : 0);
    check_launch("accum_k");
    launch_df(st, dsteps, d_d);
    resid_k<<<gsz(En), 256, 0, st>>>(En, dB, dr);
    check_launch("resid_k");
    colnorm_seg_k<<<C, 256, 0, st>>>(d_c, dr, norms + C);
    check_launch("colnorm_seg_k");
    SLU_CHECK_CUDA(
        cudaMemcpyAsync(host + C, norms + C, 8 * (size_t)C, cudaMemcpyDeviceToHost, st));
  };

  seg_copy_k<<<cgrid, 256, 0, st>>>(d_i);
  check_launch("seg_copy_k");
  iteration(true);
  int it = 1;
  double worst = 0.0;
  std::vector<double> member(m, 0.0);
  for (;;) {
    if (it < 2 && it < maxit && tol < 1e-6) {  // first correction without a check
      iteration(false);
      ++it;
      continue;
    }
    SLU_CHECK_CUDA(cudaStreamSynchronize(st));
    worst = 0.0;
    int col = 0;
    for (int j = 0; j < m; ++j) {
      double w = 0.0;
      for (int q = 0; q < cm[j]; ++q, ++col) {
        const double bj = host[col], rj = host[C + col];
        w = std::max(w, std::sqrt(rj) / (bj > 0 ? std::sqrt(bj) : 1.0));
      }
      member[j] = w;
      worst = std::max(worst, w);
    }
    if (worst <= tol || it >= maxit) break;
    iteration(false);
    ++it;
  }
  h.readback.release(st);
  seg_copy_k<<<cgrid, 256, 0, st>>>(d_o);
  check_launch("seg_copy_k");
  if (iters) *iters = it;
  if (relres)
    for (int j = 0; j < m; ++j) relres[idx[j]] = member[j];
  if (worst > tol) throw Error(SLU_ERR_NOT_CONVERGED, "refinement did not reach the tolerance");
}

}  // namespace slu
