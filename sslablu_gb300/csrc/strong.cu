// Strong-admissibility HBS: compression from sketches and apply.
//
// The operator (matAssembly/HBS/HBStorch_strong.py, HBSMAT 908-1310) is
//   A = U B V^T + E  per level, B recursively the next level's operator,
// where E is block sparse: the near-field tiles E_ij, j in NF(i) = the
// level adjacency of block i plus i itself.  Compression (leaf level first):
//   * per block i, the near-field Omega stack S_nf = [Om_j : j in NF(i)]
//     (m = |NF(i)| b rows of s samples) is factored by a Householder QR of
//     S_nf^T with the rows of Y_i carried along: one pass yields R, the
//     projection coefficients P = Y_i Q and Y_i Q_perp (_factor_nf,
//     _rowspace, 261-301);
//   * U_i = leading left singular vectors of Y_i Q_perp -- those of
//     Y_i (I - Q Q^T) (_range_via_projection, 318-332);
//   * term 1 of the tiles, (I - U_i U_i^T) A_ij = [(P - U_i U_i^T P) R^-T]_j
//     (the right solve against the stack, _pinv_rhs, 303-315);
//   * the same on the Psi stacks gives V_j and X2 = (Z_j - V_j V_j^T Z_j)
//     pinv(S_nf(Psi)); term 2 adds U_i U_i^T [X2]_i^T to tile (i, j)
//     (compute_bases_and_E_strong, 687-797);
//   * sketch reduction Y <- U^T (Y - E Om), Z <- V^T (Z - E^T Psi),
//     Om <- V^T Om, Psi <- U^T Psi, children stacked into their parent
//     (constructHBS, 1060-1080);
//   * when no block of a level has a far field, the dense base
//     B = Y pinv(Om) through the same QR (compute_final_E, 897-906).
// Blocks of one level are grouped by near-field size (NearField, 199-246):
// one group's stacks factor in one batched blocked QR (qr_blocked: panels +
// compact-WY GEMM updates over all SMs), one batched Jacobi SVD, batched
// GEMMs and triangular solves.  The QR path is upstream's fast path; its
// truncated-SVD fallback (taken upstream when a stack is numerically rank
// deficient, min |R_ii| <= 1e-12 max |R_ii|, or wider than s) is not built:
// such a stack is reported as an error.
//
// Apply (_sweep, 1232-1293): x gathered into tree order, VV_{t+1} =
// V_t^T VV_t (children stacked), u = B VV_top, then per level
// u_t = U_t u_{t+1} + E_t VV_t, scattered back; mode T swaps U and V and
// uses E^T and B^T.  All float64.
#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "abi_types.cuh"
#include "hbs.cuh"

namespace slu {
namespace strong {

struct SLevel {
  int Nb = 0, b = 0, r = 0;
  int nnz = 0;
  DevBuf U, V, tiles;          // Nb*b x r, Nb*b x r, nnz x b x b
  DevBuf rc;                   // int2 (row, col) of every tile
  std::vector<int> trow, tcol; // tile t = (trow[t], tcol[t]), sorted by (row, col)
};

struct Op {
  long long N = 0;
  int Nb0 = 0, fac = 2, nl = 0;
  DevBuf perm;                 // int64[N]: tree position i holds caller row perm[i]
  std::vector<SLevel> lv;
  int nB = 0;
  DevBuf B;                    // dense base, nB x nB
  int rk = 0, s = 0;
  long long qr_stacks = 0;     // near-field stacks factored (upstream's factor_stats)
  bool built = false;
  std::mutex mu;
};

// ---------------------------------------------------------------- kernels
// dst item d = g * per + q (gridDim.y) <- block idx[d] of src0 (q < k1) or
// src1 (q >= k1), blk doubles each.
__global__ void gather_blocks_kernel(const double* __restrict__ src0,
                                     const double* __restrict__ src1,
                                     const int* __restrict__ idx, int per, int k1, long long blk,
                                     double* __restrict__ dst) {
  const long long d = blockIdx.y;
  const int q = (int)(d % per);
  const double* s = (q < k1 ? src0 : src1) + (long long)__ldg(idx + d) * blk;
  double* o = dst + d * blk;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < blk;
       e += (long long)gridDim.x * blockDim.x)
    o[e] = s[e];
}

// dst block idx[g] <- src block g.
__global__ void scatter_blocks_kernel(const double* __restrict__ src, const int* __restrict__ idx,
                                      long long blk, double* __restrict__ dst) {
  const long long g = blockIdx.y;
  const double* s = src + g * blk;
  double* o = dst + (long long)__ldg(idx + g) * blk;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < blk;
       e += (long long)gridDim.x * blockDim.x)
    o[e] = s[e];
}

// Tiles of pair p = g * k + a (gridDim.y): mode 0 copies column block a of
// X_g (b x kb, row-major), mode 1 adds the pair-ordered b x b block p.
__global__ void tile_put_kernel(int mode, const double* __restrict__ src,
                                const int* __restrict__ tid, int k, int b, int kb,
                                double* __restrict__ tiles) {
  const long long p = blockIdx.y;
  const long long g = p / k;
  const int a = (int)(p - g * k);
  double* t = tiles + (long long)__ldg(tid + p) * b * b;
  const long long bb = (long long)b * b;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < bb;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / b), c = (int)(e - (long long)r * b);
    if (mode == 0)
      t[e] = src[g * b * kb + (long long)r * kb + (long long)a * b + c];
    else
      t[e] += src[p * bb + e];
  }
}

// R's diagonal of every factored stack (column-major, ldw): counts the
// stacks with min |R_ii| <= 1e-12 max |R_ii| (upstream's QR-path test).
__global__ void diag_check_kernel(const double* __restrict__ W, int ldw, long long sW, int m,
                                  int batch, int* __restrict__ bad) {
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= batch) return;
  const double* w = W + (long long)g * sW;
  double mn = INFINITY, mx = 0.0;
  for (int i = lane; i < m; i += 32) {
    const double d = fabs(w[(long long)i * ldw + i]);
    mn = fmin(mn, d);
    mx = fmax(mx, d);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0 && !(mn > 1e-12 * mx)) atomicAdd(bad, 1);
}

// out_dst(t) (b x c, ld ldo) += alpha * op(T_t) X_src(t) for every tile t
// (op = identity, dst = row(t), src = col(t); for trans the transpose,
// dst = col(t), src = row(t)): one CTA per (64 x 64 output tile, tile t),
// so a level's products spread over all SMs; the contributions of the
// tiles of one block row meet in float64 atomic adds (their order, and so
// the last bit of the sum, may vary between runs).  16 x 16 threads, 4 x 4
// outputs each, K staged through shared memory 16 at a time.
constexpr int kBT = 64, kBK = 16;
__global__ void __launch_bounds__(256)
bsr_mm_kernel(int trans, int b, int c, double alpha, const double* __restrict__ tiles,
              const int2* __restrict__ rc, const double* __restrict__ X, int ldx,
              double* __restrict__ out, int ldo) {
  __shared__ double As[kBK][kBT + 1];
  __shared__ double Bs[kBK][kBT];
  const int t = blockIdx.z;
  const int r0 = blockIdx.y * kBT, c0 = blockIdx.x * kBT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int2 ij = rc[t];
  const int dst = trans ? ij.y : ij.x, src = trans ? ij.x : ij.y;
  const double* T = tiles + (long long)t * b * b;
  const double* Xs = X + (long long)src * b * ldx;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < b; k0 += kBK) {
    for (int q = threadIdx.x; q < kBK * kBT; q += 256) {
      const int kk = q / kBT, rr = q - kk * kBT;   // A(r0 + rr, k0 + kk)
      const int row = r0 + rr, col = k0 + kk;
      double v = 0.0;
      if (row < b && col < b) v = trans ? T[(long long)col * b + row] : T[(long long)row * b + col];
      As[kk][rr] = v;
      const int cc = c0 + rr;                      // X(k0 + kk, c0 + rr)
      Bs[kk][rr] = (col < b && cc < c) ? Xs[(long long)col * ldx + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      double a[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = As[kk][ty + 16 * u];
        bv[u] = Bs[kk][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
  double* o = out + (long long)dst * b * ldo;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int row = r0 + ty + 16 * u;
    if (row >= b) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int col = c0 + tx + 16 * v;
      if (col < c) atomicAdd(o + (long long)row * ldo + col, alpha * acc[u][v]);
    }
  }
}

// dst row i (ld ldd) <- src row (sidx ? sidx[i] : i), or with didx the
// scatter dst row didx[i] <- src row i.
__global__ void permute_rows_kernel(long long rows, int c, const double* __restrict__ src,
                                    int lds, const int64_t* __restrict__ sidx,
                                    double* __restrict__ dst, int ldd,
                                    const int64_t* __restrict__ didx) {
  const long long n = rows * c;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / c;
    const int j = (int)(e - i * c);
    const long long si = sidx ? __ldg(sidx + i) : i;
    const long long di = didx ? __ldg(didx + i) : i;
    dst[di * ldd + j] = src[si * lds + j];
  }
}

unsigned grid1(long long n) {
  return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 65535));
}

void gather_blocks(cudaStream_t st, const double* src0, const double* src1, const int* idx,
                   int items, int per, int k1, long long blk, double* dst) {
  if (items <= 0) return;
  dim3 grid((unsigned)std::min<long long>((blk + 255) / 256, 64), (unsigned)items);
  gather_blocks_kernel<<<grid, 256, 0, st>>>(src0, src1, idx, per, k1, blk, dst);
  check_launch("gather_blocks_kernel");
}

void scatter_blocks(cudaStream_t st, const double* src, const int* idx, int items, long long blk,
                    double* dst) {
  if (items <= 0) return;
  dim3 grid((unsigned)std::min<long long>((blk + 255) / 256, 64), (unsigned)items);
  scatter_blocks_kernel<<<grid, 256, 0, st>>>(src, idx, blk, dst);
  check_launch("scatter_blocks_kernel");
}

void tile_put(cudaStream_t st, int mode, const double* src, const int* tid, int pairs, int k,
              int b, int kb, double* tiles) {
  if (pairs <= 0) return;
  dim3 grid((unsigned)std::min<long long>(((long long)b * b + 255) / 256, 32), (unsigned)pairs);
  tile_put_kernel<<<grid, 256, 0, st>>>(mode, src, tid, k, b, kb, tiles);
  check_launch("tile_put_kernel");
}

void bsr_mm(cudaStream_t st, bool trans, const SLevel& l, int c, double alpha, const double* X,
            int ldx, double* out, int ldo) {
  if (l.nnz == 0 || c <= 0) return;
  SLU_REQUIRE(l.nnz <= 65535, "strong HBS: more than 65535 near-field tiles on a level");
  dim3 grid((unsigned)((c + kBT - 1) / kBT), (unsigned)((l.b + kBT - 1) / kBT), (unsigned)l.nnz);
  bsr_mm_kernel<<<grid, 256, 0, st>>>(trans ? 1 : 0, l.b, c, alpha, l.tiles.as<double>(),
                                      l.rc.as<int2>(), X, ldx, out, ldo);
  check_launch("bsr_mm_kernel");
}

void permute_rows(cudaStream_t st, long long rows, int c, const double* src, int lds,
                  const int64_t* sidx, double* dst, int ldd, const int64_t* didx) {
  if (rows <= 0 || c <= 0) return;
  permute_rows_kernel<<<grid1(rows * c), 256, 0, st>>>(rows, c, src, lds, sidx, dst, ldd, didx);
  check_launch("permute_rows_kernel");
}

template <class T>
void upload(cudaStream_t st, DevBuf& d, const std::vector<T>& h) {
  d.alloc(std::max<size_t>(1, h.size()) * sizeof(T), st);
  if (!h.empty())
    SLU_CHECK_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

}  // namespace strong
}  // namespace slu

namespace slu {
namespace strong {

// Near-field structure of one level from the caller's CSR (NF(i) sorted,
// containing i, symmetric): tiles, row / column CSR, groups by size.
struct Group {
  int k = 0;
  std::vector<int> ranks;
};
struct Plan {
  std::vector<std::vector<int>> nf;
  std::vector<Group> groups;
  std::vector<int> trow, tcol;
  std::vector<int> tile_of_row_start;   // tiles of row i start here (sorted rows)
};

Plan plan_level(int Nb, const int* ptr, const int* idx) {
  Plan P;
  P.nf.resize(Nb);
  for (int i = 0; i < Nb; ++i) {
    SLU_REQUIRE(ptr[i + 1] >= ptr[i], "strong HBS: bad near-field CSR");
    std::vector<int>& v = P.nf[i];
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
      SLU_REQUIRE(idx[e] >= 0 && idx[e] < Nb, "strong HBS: near-field index out of range");
      v.push_back(idx[e]);
    }
    std::sort(v.begin(), v.end());
    SLU_REQUIRE(std::adjacent_find(v.begin(), v.end()) == v.end(),
                "strong HBS: repeated near-field entry");
    SLU_REQUIRE(std::binary_search(v.begin(), v.end(), i),
                "strong HBS: a block's near field must contain the block");
  }
  for (int i = 0; i < Nb; ++i)
    for (int j : P.nf[i])
      SLU_REQUIRE(std::binary_search(P.nf[j].begin(), P.nf[j].end(), i),
                  "strong HBS: the adjacency must be symmetric");
  P.tile_of_row_start.resize(Nb + 1, 0);
  for (int i = 0; i < Nb; ++i) {
    P.tile_of_row_start[i] = (int)P.trow.size();
    for (int j : P.nf[i]) {
      P.trow.push_back(i);
      P.tcol.push_back(j);
    }
  }
  P.tile_of_row_start[Nb] = (int)P.trow.size();
  std::vector<int> ks;
  for (int i = 0; i < Nb; ++i) ks.push_back((int)P.nf[i].size());
  std::vector<int> uk = ks;
  std::sort(uk.begin(), uk.end());
  uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
  for (int k : uk) {
    Group g;
    g.k = k;
    for (int i = 0; i < Nb; ++i)
      if (ks[i] == k) g.ranks.push_back(i);
    P.groups.push_back(std::move(g));
  }
  return P;
}

int tile_index(const Plan& P, int i, int j) {
  const std::vector<int>& v = P.nf[i];
  return P.tile_of_row_start[i] + (int)(std::lower_bound(v.begin(), v.end(), j) - v.begin());
}

// One pass (Omega / Y or Psi / Z) over a group: basis into Bg (G x b x r),
// the right-solved residual sketch into Xb (G x b x kb).  Returns nothing;
// failures of the QR test are counted in bad.
struct GroupWs {
  double *WS, *tau, *tau2, *qr, *Bg, *sv, *T1, *Xb, *G2, *T2, *Cor;
  int *idx, *tid;
};

void group_pass(cudaStream_t st, int b, int r, int s, const Group& g, const double* Omk, const double* Ysk, const GroupWs& w, int* info, int* bad) {
  const int G = (int)g.ranks.size(), k = g.k, m = k * b;
  const long long sW = (long long)(m + b) * s;
  gather_blocks(st, Omk, Ysk, w.idx, G * (k + 1), k + 1, k, (long long)b * s, w.WS);
  qr_blocked(st, s, m, m + b, w.WS, s, sW, w.tau, m, G, w.qr);
  diag_check_kernel<<<(G + 7) / 8, 256, 0, st>>>(w.WS, s, sW, m, G, bad);
  check_launch("diag_check_kernel");
  // basis: left singular vectors of Y_i Q_perp (b x (s - m))
  double* perp = w.WS + (long long)m * s + m;
  const int jc = s - m;
  if (jc > b) {
    panel_qr(st, jc, b, b, perp, s, sW, w.tau2, b, G);
    jacobi_left_sv(st, b, b, perp, s, sW, r, w.Bg, r, (long long)b * r, w.sv, b, G, info, true);
  } else {
    jacobi_left_sv(st, b, jc, perp, s, sW, r, w.Bg, r, (long long)b * r, w.sv, b, G, info, false);
  }
  // (P - B B^T P) R^-T, P = Y_i Q (b x m, ld s)
  const double* Pp = w.WS + (long long)m * s;
  const long long br = (long long)b * r, rm = (long long)r * m, bm = (long long)b * m;
  gemm_batched<double>(st, true, false, r, m, b, 1.0, w.Bg, r, br, 0, Pp, s, sW, 0, 0.0, w.T1, m,
                       rm, 0, G);
  copy_batched<double>(st, b, m, Pp, s, sW, 0, w.Xb, m, bm, 0, G);
  gemm_batched<double>(st, false, false, b, m, r, -1.0, w.Bg, r, br, 0, w.T1, m, rm, 0, 1.0, w.Xb,
                       m, bm, 0, G);
  trsm_upper<double>(st, false, m, w.WS, 1, s, sW, w.Xb, 1, m, bm, b, G);
}

}  // namespace strong

using strong::SLevel;
using strong::Op;

void strong_compress(Handle& h, Op& S, int rk, int s, const double* Om, const double* Psi,
                     const double* Y, const double* Z, int nlev, const int* nb,
                     const int* nf_ptr, const int* nf_idx) {
  using namespace strong;
  cudaStream_t st = h.stream;
  const long long N = S.N;
  SLU_REQUIRE(rk >= 1 && s >= 1 && nlev >= 0, "strong HBS: bad rank, sample count or levels");
  // level geometry (HBStorch_strong.py:1033-1100): leaf blocks of nl rows,
  // rank min(rk, nl); above, fac children of rank r stack into b = fac r rows
  std::vector<Plan> plans;
  std::vector<SLevel> lv(nlev);
  {
    int Nb = S.Nb0, b = S.nl;
    long long off_p = 0, off_i = 0;
    for (int t = 0; t < nlev; ++t) {
      SLU_REQUIRE(nb[t] == Nb, "strong HBS: level " + std::to_string(t) + " has " +
                                   std::to_string(nb[t]) + " blocks, the tree gives " +
                                   std::to_string(Nb));
      plans.push_back(plan_level(Nb, nf_ptr + off_p, nf_idx + off_i));
      off_i += nf_ptr[off_p + Nb];
      off_p += Nb + 1;
      lv[t].Nb = Nb;
      lv[t].b = b;
      lv[t].r = std::min(rk, b);
      SLU_REQUIRE(Nb % S.fac == 0 || Nb == 1, "strong HBS: blocks do not pair into parents");
      b = S.fac * lv[t].r;
      Nb /= S.fac;
      SLU_REQUIRE(Nb >= 1, "strong HBS: more compressed levels than the tree has");
    }
  }
  // workspace: the sketches (current and next, 4 arrays each) and the
  // largest group's buffers
  const size_t Ns = (size_t)N * s;
  size_t gmax = 0, qmax = 0;
  for (int t = 0; t < nlev; ++t) {
    const SLevel& l = lv[t];
    for (const Group& g : plans[t].groups) {
      const size_t G = g.ranks.size(), m = (size_t)g.k * l.b, b = l.b, r = l.r;
      SLU_REQUIRE((int)m <= s, "strong HBS: a near-field stack has more rows (" +
                                   std::to_string(m) + ") than samples (" + std::to_string(s) +
                                   "); upstream's SVD fallback for that case is not built");
      SLU_REQUIRE(r <= (size_t)s - m, "strong HBS: rank exceeds the samples left after the "
                                      "near field");
      const size_t need = G * (m + b) * s + G * m + G * b + G * b * r + G * b + G * r * m +
                          G * b * m + 3 * G * g.k * b * b + G * g.k * b * r + 64 * 12;
      gmax = std::max(gmax, need);
      qmax = std::max(qmax, qr_blocked_ws_elems(s, (int)(m + b), (int)G));
    }
  }
  long long nB = nlev == 0 ? N : (long long)lv[nlev - 1].Nb * lv[nlev - 1].r;
  SLU_REQUIRE(nB <= s, "strong HBS: the dense base (" + std::to_string(nB) +
                           " rows) is larger than the sample count; upstream's pinv fallback "
                           "for that case is not built");
  const size_t base_need = 2 * (size_t)nB * s + (size_t)nB + 64;
  qmax = std::max(qmax, qr_blocked_ws_elems(s, (int)(2 * nB), 1));
  const size_t total = 8 * (8 * Ns + std::max(gmax, base_need) + qmax) + 64 * 1024;
  h.ws.reserve(total, st);
  double* cur[4];
  double* nxt[4];
  for (int a = 0; a < 4; ++a) cur[a] = h.ws.take<double>(Ns);
  for (int a = 0; a < 4; ++a) nxt[a] = h.ws.take<double>(Ns);
  double* gbuf = h.ws.take<double>(std::max(gmax, base_need));
  double* qrws = h.ws.take<double>(qmax);
  SLU_CHECK_CUDA(cudaMemcpyAsync(cur[0], Om, 8 * Ns, cudaMemcpyDeviceToDevice, st));
  SLU_CHECK_CUDA(cudaMemcpyAsync(cur[1], Psi, 8 * Ns, cudaMemcpyDeviceToDevice, st));
  SLU_CHECK_CUDA(cudaMemcpyAsync(cur[2], Y, 8 * Ns, cudaMemcpyDeviceToDevice, st));
  SLU_CHECK_CUDA(cudaMemcpyAsync(cur[3], Z, 8 * Ns, cudaMemcpyDeviceToDevice, st));
  int* info = h.info.as<int>();
  SLU_CHECK_CUDA(cudaMemsetAsync(info, 0, 64 * sizeof(int), st));
  int* bad = info + 8;
  long long stacks = 0;
  for (int t = 0; t < nlev; ++t) {
    SLevel& l = lv[t];
    const Plan& P = plans[t];
    const int Nb = l.Nb, b = l.b, r = l.r;
    l.nnz = (int)P.trow.size();
    l.trow = P.trow;
    l.tcol = P.tcol;
    l.U.alloc(8 * (size_t)Nb * b * r, st);
    l.V.alloc(8 * (size_t)Nb * b * r, st);
    l.tiles.alloc(8 * (size_t)l.nnz * b * b, st);
    {
      std::vector<int2> rc(l.nnz);
      for (int t2 = 0; t2 < l.nnz; ++t2) rc[t2] = make_int2(P.trow[t2], P.tcol[t2]);
      upload(st, l.rc, rc);
    }
    // pass 0: Omega stacks, Y -> U and term 1; pass 1: Psi stacks, Z -> V
    // and term 2 (needs every U of the level, so all groups of pass 0 first)
    for (int pass = 0; pass < 2; ++pass) {
      const double* Omk = cur[pass == 0 ? 0 : 1];
      const double* Ysk = cur[pass == 0 ? 2 : 3];
      double* basis = (pass == 0 ? l.U : l.V).as<double>();
      for (const Group& g : P.groups) {
        const int G = (int)g.ranks.size(), k = g.k, m = k * b;
        GroupWs w{};
        double* p = gbuf;
        auto take = [&](size_t n) {
          double* q = p;
          p += (n + 31) & ~size_t(31);
          return q;
        };
        w.WS = take((size_t)G * (m + b) * s);
        w.tau = take((size_t)G * m);
        w.tau2 = take((size_t)G * b);
        w.Bg = take((size_t)G * b * r);
        w.sv = take((size_t)G * b);
        w.T1 = take((size_t)G * r * m);
        w.Xb = take((size_t)G * b * m);
        w.G2 = take((size_t)G * k * b * r);
        w.T2 = take((size_t)G * k * r * b);
        w.Cor = take((size_t)G * k * b * b);
        w.qr = qrws;
        // index tables: stack blocks (NF(i) then i), tiles of the pairs
        std::vector<int> hidx, htid, hnf;
        for (int i : g.ranks) {
          for (int j : P.nf[i]) hidx.push_back(j);
          hidx.push_back(i);
          for (int j : P.nf[i]) {
            hnf.push_back(j);
            htid.push_back(pass == 0 ? tile_index(P, i, j) : tile_index(P, j, i));
          }
        }
        DevBuf didx, dtid, dnf, drank;
        upload(st, didx, hidx);
        upload(st, dtid, htid);
        upload(st, dnf, hnf);
        upload(st, drank, g.ranks);
        w.idx = didx.as<int>();
        group_pass(st, b, r, s, g, Omk, Ysk, w, info, bad);
        scatter_blocks(st, w.Bg, drank.as<int>(), G, (long long)b * r, basis);
        if (pass == 0) {
          tile_put(st, 0, w.Xb, dtid.as<int>(), G * k, k, b, m, l.tiles.as<double>());
        } else {
          // term 2: tile (i, j) += U_i U_i^T [X2_j]_i^T for i in NF(j)
          gather_blocks(st, l.U.as<double>(), l.U.as<double>(), dnf.as<int>(), G * k, k, k,
                        (long long)b * r, w.G2);
          const long long br = (long long)b * r, bb = (long long)b * b;
          gemm_batched<double>(st, true, true, r, b, b, 1.0, w.G2, r, br, k * br, w.Xb, m, b,
                               (long long)b * m, 0.0, w.T2, b, (long long)r * b,
                               (long long)k * r * b, k, G);
          gemm_batched<double>(st, false, false, b, b, r, 1.0, w.G2, r, br, k * br, w.T2, b,
                               (long long)r * b, (long long)k * r * b, 0.0, w.Cor, b, bb, k * bb,
                               k, G);
          tile_put(st, 1, w.Cor, dtid.as<int>(), G * k, k, b, m, l.tiles.as<double>());
        }
        stacks += G;
      }
    }
    // a rank-deficient stack leaves non-finite tiles: stop at this level
    // rather than carry them into the next level's sketches
    {
      int hb = 0;
      SLU_CHECK_CUDA(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
      stream_wait(st);
      SLU_REQUIRE(hb == 0, "strong HBS: " + std::to_string(hb) +
                               " near-field stack(s) of level " + std::to_string(t) +
                               " numerically rank deficient (min |R_ii| <= 1e-12 max |R_ii|); "
                               "upstream's truncated-SVD fallback for that case is not built");
    }
    // sketch reduction (HBStorch_strong.py:1060-1080)
    bsr_mm(st, false, l, s, -1.0, cur[0], s, cur[2], s);   // Y -= E Om
    bsr_mm(st, true, l, s, -1.0, cur[1], s, cur[3], s);    // Z -= E^T Psi
    const long long br = (long long)b * r, bs = (long long)b * s, rs = (long long)r * s;
    const double* Ut = l.U.as<double>();
    const double* Vt = l.V.as<double>();
    gemm_batched<double>(st, true, false, r, s, b, 1.0, Vt, r, br, 0, cur[0], s, bs, 0, 0.0,
                         nxt[0], s, rs, 0, Nb);
    gemm_batched<double>(st, true, false, r, s, b, 1.0, Ut, r, br, 0, cur[1], s, bs, 0, 0.0,
                         nxt[1], s, rs, 0, Nb);
    gemm_batched<double>(st, true, false, r, s, b, 1.0, Ut, r, br, 0, cur[2], s, bs, 0, 0.0,
                         nxt[2], s, rs, 0, Nb);
    gemm_batched<double>(st, true, false, r, s, b, 1.0, Vt, r, br, 0, cur[3], s, bs, 0, 0.0,
                         nxt[3], s, rs, 0, Nb);
    for (int a = 0; a < 4; ++a) std::swap(cur[a], nxt[a]);
  }
  // dense base B = Y pinv(Om) (compute_final_E, 897-906)
  {
    double* WSb = gbuf;
    double* taub = gbuf + 2 * (size_t)nB * s;
    SLU_CHECK_CUDA(cudaMemcpyAsync(WSb, cur[0], 8 * (size_t)nB * s, cudaMemcpyDeviceToDevice, st));
    SLU_CHECK_CUDA(cudaMemcpyAsync(WSb + (size_t)nB * s, cur[2], 8 * (size_t)nB * s,
                                   cudaMemcpyDeviceToDevice, st));
    qr_blocked(st, s, (int)nB, (int)(2 * nB), WSb, s, 0, taub, 0, 1, qrws);
    diag_check_kernel<<<1, 256, 0, st>>>(WSb, s, 0, (int)nB, 1, bad);
    check_launch("diag_check_kernel");
    S.B.alloc(8 * (size_t)nB * nB, st);
    copy_batched<double>(st, (int)nB, (int)nB, WSb + (size_t)nB * s, s, 0, 0, S.B.as<double>(),
                         (int)nB, 0, 0, 1);
    trsm_upper<double>(st, false, (int)nB, WSb, 1, s, 0, S.B.as<double>(), 1, nB, 0, (int)nB, 1);
  }
  int hinfo[16];
  SLU_CHECK_CUDA(cudaMemcpyAsync(hinfo, info, sizeof(hinfo), cudaMemcpyDeviceToHost, st));
  stream_wait(st);
  SLU_REQUIRE(hinfo[0] == 0, "strong HBS: a Jacobi SVD of a projected sketch did not converge");
  SLU_REQUIRE(hinfo[8] == 0, "strong HBS: " + std::to_string(hinfo[8]) +
                                 " near-field stack(s) numerically rank deficient "
                                 "(min |R_ii| <= 1e-12 max |R_ii|); upstream's truncated-SVD "
                                 "fallback for that case is not built");
  S.lv = std::move(lv);
  S.nB = (int)nB;
  S.rk = rk;
  S.s = s;
  S.qr_stacks = stacks;
  S.built = true;
}

size_t strong_apply_scratch(const Op& S, int c) {
  size_t e = 3 * (size_t)S.N * c;
  for (const SLevel& l : S.lv) e += (size_t)l.Nb * l.r * c + 32;
  return e + 64;
}

void strong_apply(Handle& h, const Op& S, bool trans, const double* X, int ldx, double* Yout,
                  int ldy, int c) {
  using namespace strong;
  SLU_REQUIRE(S.built, "strong HBS: not compressed");
  cudaStream_t st = h.stream;
  const int nlev = (int)S.lv.size();
  h.ws.reserve(8 * strong_apply_scratch(S, c) + 64 * 1024, st);
  std::vector<double*> VV(nlev + 1);
  VV[0] = h.ws.take<double>((size_t)S.N * c);
  for (int t = 0; t < nlev; ++t) VV[t + 1] = h.ws.take<double>((size_t)S.lv[t].Nb * S.lv[t].r * c);
  double* u[2] = {h.ws.take<double>((size_t)S.N * c), h.ws.take<double>((size_t)S.N * c)};
  const int64_t* perm = S.perm.as<int64_t>();
  permute_rows(st, S.N, c, X, ldx, perm, VV[0], c, nullptr);
  for (int t = 0; t < nlev; ++t) {
    const SLevel& l = S.lv[t];
    const double* D = (trans ? l.U : l.V).as<double>();
    gemm_batched<double>(st, true, false, l.r, c, l.b, 1.0, D, l.r, (long long)l.b * l.r, 0,
                         VV[t], c, (long long)l.b * c, 0, 0.0, VV[t + 1], c, (long long)l.r * c,
                         0, l.Nb);
  }
  int cur = 0;
  gemm_batched<double>(st, trans, false, S.nB, c, S.nB, 1.0, S.B.as<double>(), S.nB, 0, 0,
                       VV[nlev], c, 0, 0, 0.0, u[cur], c, 0, 0, 1);
  for (int t = nlev - 1; t >= 0; --t) {
    const SLevel& l = S.lv[t];
    const double* D = (trans ? l.V : l.U).as<double>();
    gemm_batched<double>(st, false, false, l.b, c, l.r, 1.0, D, l.r, (long long)l.b * l.r, 0,
                         u[cur], c, (long long)l.r * c, 0, 0.0, u[cur ^ 1], c,
                         (long long)l.b * c, 0, l.Nb);
    cur ^= 1;
    bsr_mm(st, trans, l, c, 1.0, VV[t], c, u[cur], c);
  }
  permute_rows(st, S.N, c, u[cur], c, nullptr, Yout, ldy, perm);
}

}  // namespace slu

// ---------------------------------------------------------------- C ABI
struct slu_strong_s {
  slu::strong::Op S;
};

extern "C" int slu_strong_create(slu_handle_t h, long long N, int nleaves, int fac,
                                 const int64_t* perm_host, slu_strong_t* out) {
  return slu::guard_call(h, [&] {
    using namespace slu;
    SLU_REQUIRE(h && out, "null argument");
    SLU_REQUIRE(N > 0 && nleaves >= 1 && (fac == 2 || fac == 4), "bad strong HBS geometry");
    SLU_REQUIRE(N % nleaves == 0, "N must be a multiple of the leaf count (uniform leaves)");
    auto p = std::make_unique<slu_strong_s>();
    p->S.N = N;
    p->S.Nb0 = nleaves;
    p->S.fac = fac;
    p->S.nl = (int)(N / nleaves);
    std::vector<int64_t> perm(N);
    std::vector<char> seen(N, 0);
    for (long long i = 0; i < N; ++i) {
      const int64_t v = perm_host ? perm_host[i] : i;
      SLU_REQUIRE(v >= 0 && v < N && !seen[v], "perm is not a permutation of 0..N-1");
      seen[v] = 1;
      perm[i] = v;
    }
    strong::upload(h->h.stream, p->S.perm, perm);
    slu::stream_wait(h->h.stream);
    *out = p.release();
  });
}

extern "C" int slu_strong_destroy(slu_strong_t op) {
  return slu::guard_call(nullptr, [&] { delete op; });
}

extern "C" int slu_strong_compress(slu_handle_t h, slu_strong_t op, int rk, int s,
                                   const double* Om, const double* Psi, const double* Y,
                                   const double* Z, int nlev, const int* nb, const int* nf_ptr,
                                   const int* nf_idx) {
  return slu::guard_call(h, [&] {
    SLU_REQUIRE(h && op && Om && Psi && Y && Z, "null argument");
    SLU_REQUIRE(nlev == 0 || (nb && nf_ptr && nf_idx), "null near-field tables");
    std::lock_guard<std::mutex> lock(op->S.mu);
    op->S.built = false;
    slu::strong_compress(h->h, op->S, rk, s, Om, Psi, Y, Z, nlev, nb, nf_ptr, nf_idx);
  });
}

extern "C" int slu_strong_apply(slu_handle_t h, slu_strong_t op, int trans, const double* X,
                                int ldx, double* Y, int ldy, int nrhs) {
  return slu::guard_call(h, [&] {
    SLU_REQUIRE(h && op && X && Y, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldx >= nrhs && ldy >= nrhs, "bad right-hand-side shape");
    SLU_REQUIRE(static_cast<const void*>(X) != static_cast<const void*>(Y),
                "strong HBS apply: input and output must be different buffers");
    slu::strong_apply(h->h, op->S, trans != 0, X, ldx, Y, ldy, nrhs);
  });
}

extern "C" int slu_strong_info(slu_strong_t op, int what, int level, long long* out) {
  return slu::guard_call(nullptr, [&] {
    SLU_REQUIRE(op && out, "null argument");
    const slu::strong::Op& S = op->S;
    SLU_REQUIRE(S.built || what == 0, "strong HBS: not compressed");
    const int nl = (int)S.lv.size();
    auto L = [&]() -> const slu::strong::SLevel& {
      SLU_REQUIRE(level >= 0 && level < nl, "level out of range");
      return S.lv[level];
    };
    switch (what) {
      case 0: *out = S.built ? nl : -1; break;       // compressed levels
      case 1: *out = L().Nb; break;
      case 2: *out = L().b; break;
      case 3: *out = L().r; break;
      case 4: *out = L().nnz; break;
      case 5: *out = S.nB; break;                    // rows of the dense base
      case 6: *out = S.qr_stacks; break;             // near-field stacks factored
      case 7: {                                      // bytes of U, V, E and the base
        // (tiles with their int64 row / column indices, as upstream counts)
        long long b = 8LL * S.nB * S.nB;
        for (const auto& l : S.lv)
          b += 8LL * (2LL * l.Nb * l.b * l.r + (long long)l.nnz * l.b * l.b) + 16LL * l.nnz;
        *out = b;
        break;
      }
      default: SLU_REQUIRE(false, "unknown strong HBS query");
    }
  });
}

extern "C" int slu_strong_export(slu_handle_t h, slu_strong_t op, int what, int level,
                                 void* dst) {
  return slu::guard_call(h, [&] {
    using namespace slu;
    SLU_REQUIRE(h && op && dst, "null argument");
    const strong::Op& S = op->S;
    SLU_REQUIRE(S.built, "strong HBS: not compressed");
    cudaStream_t st = h->h.stream;
    if (what == 4) {   // dense base, nB x nB
      SLU_CHECK_CUDA(cudaMemcpyAsync(dst, S.B.p, 8 * (size_t)S.nB * S.nB, cudaMemcpyDefault, st));
    } else {
      SLU_REQUIRE(level >= 0 && level < (int)S.lv.size(), "level out of range");
      const strong::SLevel& l = S.lv[level];
      switch (what) {
        case 0: SLU_CHECK_CUDA(cudaMemcpyAsync(dst, l.U.p, l.U.bytes, cudaMemcpyDefault, st)); break;
        case 1: SLU_CHECK_CUDA(cudaMemcpyAsync(dst, l.V.p, l.V.bytes, cudaMemcpyDefault, st)); break;
        case 2: SLU_CHECK_CUDA(cudaMemcpyAsync(dst, l.tiles.p, l.tiles.bytes, cudaMemcpyDefault, st)); break;
        case 3: {   // tile coordinates, int32 pairs (row, col)
          std::vector<int> rc(2 * (size_t)l.nnz);
          for (int t = 0; t < l.nnz; ++t) {
            rc[2 * t] = l.trow[t];
            rc[2 * t + 1] = l.tcol[t];
          }
          std::memcpy(dst, rc.data(), rc.size() * sizeof(int));
          break;
        }
        default: SLU_REQUIRE(false, "unknown strong HBS export");
      }
    }
    stream_wait(st);
  });
}
