// Dense block-tridiagonal direct solvers on the device.
//
//   * red-black cyclic reduction: direct_solve/omsdirectsolve.py:177-333
//     (RedBlackSolver.factorize / solve / build_block_RB_solver_level)
//   * block Thomas: direct_solve/omsdirectsolve.py:48-141
//     (BlockTridiagonalSolver.factorize_helper / solve_helper)
//
// Red-black: per level, every odd block o is solved once against the stacked
// couplings [SiM_o | SiP_o] (one batched LU solve with 2m right-hand sides),
// then the new diagonal B_i and couplings A_i, C_i of every kept even block i
// come from two batched GEMMs against those solves:
//   G1 = SiM_i [T_{i-1}^{-1} SiM_{i-1} | T_{i-1}^{-1} SiP_{i-1}]
//   G2 = SiP_i [T_{i+1}^{-1} SiM_{i+1} | T_{i+1}^{-1} SiP_{i+1}]
//   A_i = -G1[:, :m],  B_i = T_i - G1[:, m:] - G2[:, :m],  C_i = -G2[:, m:].
// Periodic systems (cyclic = true, omsdirectsolve.py:207-209, 249-250,
// 269-272, 315-327) keep SiM_0 and SiP_{n-1} as the couplings to the last and
// first block: block 0's left neighbour is the last odd block at every level,
// the last kept block's right neighbour wraps to block 0 in the back
// substitution, and when a level reduces to one block its couplings to
// itself are folded into the diagonal (B_0 += A_0 + C_0).
// Upstream rebuilds each T from its LU factors (omsdirectsolve.py:31-46,314);
// this keeps T itself, the same matrix up to rounding.  The solve phase
// applies the pivot-block inverses (formed once from the LU factors) as
// GEMMs instead of triangular sweeps: the same result to rounding, and every
// block solve parallel over the block's rows.
#include "tridiag.cuh"
#include "sweep_host.cuh"

#include <algorithm>
#include <cmath>

namespace slu {
namespace {
inline double* dp(const DevBuf& b) { return b.as<double>(); }
inline int* ip(const DevBuf& b) { return b.as<int>(); }

// Inv_b = T_b^{-1} from the LU factors of nS blocks (m x m each): a batched
// LU solve against the identity.
void make_inverses(cudaStream_t st, int m, const DevBuf& LU, const DevBuf& piv, int nS,
                   DevBuf& Inv) {
  const size_t mm = (size_t)m * m;
  Inv.alloc(8 * nS * mm, st);
  identity_cols(st, m, 0, m, dp(Inv), (long long)mm, nS);
  lu_solve<double>(st, false, m, dp(LU), m, (long long)mm, ip(piv), m, dp(Inv), m,
                   (long long)mm, m, nS);
}
// Fop_j <- [I | 0 | 0] (nR blocks of m x 3m)
__global__ void rb_fop_init_kernel(int nR, int m, double* __restrict__ F) {
  const long long w = 3LL * m, total = (long long)nR * m * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long q = e % ((long long)m * w);
    const int r = (int)(q / w), c = (int)(q - r * w);
    F[e] = (c == r) ? 1.0 : 0.0;
  }
}

// F_b <- [I | 0] (nb blocks of m x w, w >= m)
__global__ void ident_wide_kernel(int nb, int m, int w, double* __restrict__ F) {
  const long long total = (long long)nb * m * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long q = e % ((long long)m * w);
    const int r = (int)(q / w), c = (int)(q - (long long)r * w);
    F[e] = (c == r) ? 1.0 : 0.0;
  }
}

// The fused solve operators of every reduction level (see RbLevel).
void build_fused_ops(cudaStream_t st, RbSolver& S) {
  const int m = S.m;
  const long long mm = (long long)m * m, w = 3LL * m;
  for (size_t l = 0; l + 1 < S.levels.size(); ++l) {
    RbLevel& P = S.levels[l];
    const int nR = P.nS / 2;
    P.Fop.alloc(8 * (size_t)nR * 3 * mm, st);
    P.Bop.alloc(8 * (size_t)nR * 3 * mm, st);
    double* F = dp(P.Fop);
    double* Bo = dp(P.Bop);
    const long long tot = (long long)nR * 3 * mm;
    rb_fop_init_kernel<<<(int)std::min<long long>((tot + 255) / 256, 8LL * num_sms()), 256, 0,
                         st>>>(nR, m, F);
    check_launch("rb_fop_init_kernel");
    // -SiM_{2j} Inv_{2j-1} (j >= 1), -SiP_{2j} Inv_{2j+1}
    if (nR > 1)
      gemm_batched<double>(st, false, false, m, m, m, -1.0, dp(P.SiM) + 2 * mm, m, 2 * mm, 0,
                           dp(P.Inv) + mm, m, 2 * mm, 0, 0.0, F + 3 * mm + m, (int)w, 3 * mm, 0,
                           nR - 1);
    gemm_batched<double>(st, false, false, m, m, m, -1.0, dp(P.SiP), m, 2 * mm, 0, dp(P.Inv) + mm,
                         m, 2 * mm, 0, 0.0, F + 2 * m, (int)w, 3 * mm, 0, nR);
    // [Inv_o | -Inv_o SiM_o | -Inv_o SiP_o]
    copy_batched<double>(st, m, m, dp(P.Inv) + mm, m, 2 * mm, 0, Bo, (int)w, 3 * mm, 0, nR);
    gemm_batched<double>(st, false, false, m, m, m, -1.0, dp(P.Inv) + mm, m, 2 * mm, 0,
                         dp(P.SiM) + mm, m, 2 * mm, 0, 0.0, Bo + m, (int)w, 3 * mm, 0, nR);
    gemm_batched<double>(st, false, false, m, m, m, -1.0, dp(P.Inv) + mm, m, 2 * mm, 0,
                         dp(P.SiP) + mm, m, 2 * mm, 0, 0.0, Bo + 2 * m, (int)w, 3 * mm, 0, nR);
  }
  S.fused = true;
}

// rb_solve with the fused operators: one step kernel per reduction level,
// one for the coarsest block, one per back-substitution level.  Level l's
// right-hand side V_l has a zero block before block 0 (read as v_{-1} next
// to the zero middle block of Fop_0); the solution X holds the blocks in
// their final order -- level l's block k is block k 2^l -- plus a zero
// block after the last (read as x_{nblk} next to the zero right block of
// the last Bop).
void rb_solve_fused(Handle& h, const RbSolver& S, double* B, int ldb, int c) {
  cudaStream_t st = h.stream;
  const int m = S.m, nblk = S.nblk, nL = (int)S.levels.size();
  const long long mc = (long long)m * c;
  size_t tot = (size_t)(nblk + 1) * mc;
  for (const RbLevel& L : S.levels) tot += (size_t)(L.nS + 1) * mc;
  h.ws.reserve(8 * tot + 8 * 256, st);
  double* base = h.ws.take<double>(tot);
  SLU_CHECK_CUDA(cudaMemsetAsync(base, 0, 8 * tot, st));
  std::vector<double*> V(nL);
  double* p = base;
  for (int l = 0; l < nL; ++l) {
    V[l] = p;
    p += (size_t)(S.levels[l].nS + 1) * mc;
  }
  double* X = p;
  copy_batched<double>(st, nblk * m, c, B, ldb, 0, 0, V[0] + mc, c, 0, 0, 1);
  auto step = [&](const double* op, long long sS, int nb, int w, int nin) {
    sweep::Step<double> s{};
    s.S = op;
    s.sS = sS;
    s.rows = m;
    s.w = w;
    s.nb = nb;
    s.c = c;
    s.nin = nin;
    s.split = m;
    for (int q = 0; q < 3; ++q) {
      s.in_ld[q] = c;
      s.in_rows[q] = m;
    }
    s.out_ld[0] = c;
    return s;
  };
  // reduction: v'_j = Fop_j [v_{2j}; v_{2j-1}; v_{2j+1}]
  for (int l = 0; l + 1 < nL; ++l) {
    const RbLevel& P = S.levels[l];
    const int nR = P.nS / 2;
    sweep::Step<double> s = step(dp(P.Fop), 3LL * m * m, nR, 3 * m, 3);
    s.in_p[0] = V[l] + mc;
    s.in_p[1] = V[l];
    s.in_p[2] = V[l] + 2 * mc;
    for (int q = 0; q < 3; ++q) s.in_blk[q] = 2LL * m;
    s.out_p[0] = V[l + 1] + mc;
    s.out_blk[0] = m;
    sweep::launch_step(st, s, "rb_reduce_step");
  }
  {  // coarsest block: x_0 = Inv v_0
    sweep::Step<double> s = step(dp(S.levels[nL - 1].Inv), 0, 1, m, 1);
    s.in_p[0] = V[nL - 1] + mc;
    s.out_p[0] = X;
    sweep::launch_step(st, s, "rb_coarse_step");
  }
  // back substitution: x_o = Bop_j [v_o; x_{o-1}; x_{o+1}], o = 2j + 1
  for (int l = nL - 2; l >= 0; --l) {
    const RbLevel& P = S.levels[l];
    const int nR = P.nS / 2;
    const long long sm = (1LL << l) * m;   // rows between level-l blocks in X
    sweep::Step<double> s = step(dp(P.Bop), 3LL * m * m, nR, 3 * m, 3);
    s.in_p[0] = V[l] + 2 * mc;
    s.in_blk[0] = 2LL * m;
    s.in_p[1] = X;
    s.in_blk[1] = 2 * sm;
    s.in_p[2] = X + 2 * sm * c;
    s.in_blk[2] = 2 * sm;
    s.out_p[0] = X + sm * c;
    s.out_blk[0] = 2 * sm;
    sweep::launch_step(st, s, "rb_back_step");
  }
  copy_batched<double>(st, nblk * m, c, X, c, 0, 0, B, ldb, 0, 0, 1);
}
}  // namespace

void rb_factor(Handle& h, RbSolver& S, int nblk, int m, const double* SiM, const double* SiP,
               const double* T, bool mixed, bool cyclic) {
  cudaStream_t st = h.stream;
  SLU_REQUIRE(nblk >= 1 && (nblk & (nblk - 1)) == 0, "red-black needs a power-of-two block count");
  SLU_REQUIRE(m >= 1, "bad block size");
  S.m = m;
  S.nblk = nblk;
  S.mixed = mixed;
  S.cyclic = cyclic;
  SLU_REQUIRE(!(cyclic && mixed), "the periodic red-black factorisation is float64 only");
  DevBuf tcws;
  if (mixed) tcws.alloc(tc_gemm_workspace_bytes(m, 2 * m, m), st);
  S.levels.clear();
  const size_t mm = (size_t)m * m;
  // level 0: copies, with the boundary couplings zeroed (omsdirectsolve.py:207-209)
  S.levels.emplace_back();
  {
    RbLevel& L0 = S.levels.back();
    L0.nS = nblk;
    L0.SiM.alloc(8 * nblk * mm, st);
    L0.SiP.alloc(8 * nblk * mm, st);
    L0.T.alloc(8 * nblk * mm, st);
    L0.LU.alloc(8 * nblk * mm, st);
    L0.piv.alloc(4 * (size_t)nblk * m, st);
    SLU_CHECK_CUDA(cudaMemcpyAsync(dp(L0.SiM), SiM, 8 * nblk * mm, cudaMemcpyDeviceToDevice, st));
    SLU_CHECK_CUDA(cudaMemcpyAsync(dp(L0.SiP), SiP, 8 * nblk * mm, cudaMemcpyDeviceToDevice, st));
    if (!cyclic) {
      SLU_CHECK_CUDA(cudaMemsetAsync(dp(L0.SiM), 0, 8 * mm, st));
      SLU_CHECK_CUDA(cudaMemsetAsync(dp(L0.SiP) + (nblk - 1) * mm, 0, 8 * mm, st));
    }
    SLU_CHECK_CUDA(cudaMemcpyAsync(dp(L0.T), T, 8 * nblk * mm, cudaMemcpyDeviceToDevice, st));
    SLU_CHECK_CUDA(cudaMemcpyAsync(dp(L0.LU), T, 8 * nblk * mm, cudaMemcpyDeviceToDevice, st));
    lu_factor(st, m, dp(L0.LU), m, mm, ip(L0.piv), m, nblk, h.info.as<int>());
    make_inverses(st, m, L0.LU, L0.piv, nblk, L0.Inv);
  }
  h.ws.reserve(8 * ((size_t)nblk / 2 * 2 * mm * 3) + 8 * 256, st);
  double* X = h.ws.take<double>(std::max<size_t>(1, (size_t)nblk / 2) * 2 * mm);  // per odd block: m x 2m
  double* G1 = h.ws.take<double>(std::max<size_t>(1, (size_t)nblk / 2) * 2 * mm);
  double* G2 = h.ws.take<double>(std::max<size_t>(1, (size_t)nblk / 2) * 2 * mm);
  int l = nblk;
  while (l > 1) {
    const RbLevel& P = S.levels.back();
    const int nR = l / 2;
    RbLevel N;
    N.nS = nR;
    N.SiM.alloc(8 * nR * mm, st);
    N.SiP.alloc(8 * nR * mm, st);
    N.T.alloc(8 * nR * mm, st);
    N.LU.alloc(8 * nR * mm, st);
    N.piv.alloc(4 * (size_t)nR * m, st);
    const long long m2 = 2 * (long long)m;
    // X_o = T_o^{-1} [SiM_o | SiP_o] for odd o, as products with the
    // inverses formed when the level was factored (GEMMs over all SMs
    // instead of substitutions)
    gemm_batched<double>(st, false, false, m, m, m, 1.0, dp(P.Inv) + mm, m, 2 * mm, 0,
                         dp(P.SiM) + mm, m, 2 * mm, 0, 0.0, X, (int)m2, 2 * mm, 0, nR);
    gemm_batched<double>(st, false, false, m, m, m, 1.0, dp(P.Inv) + mm, m, 2 * mm, 0,
                         dp(P.SiP) + mm, m, 2 * mm, 0, 0.0, X + m, (int)m2, 2 * mm, 0, nR);
    // G1_j = SiM_{2j} X_{2j-1} (j >= 1; SiM_0 is zero), G2_j = SiP_{2j} X_{2j+1}
    if (!mixed) {
      if (nR > 1)
        gemm_batched<double>(st, false, false, m, (int)m2, m, 1.0, dp(P.SiM) + 2 * mm, m, 2 * mm,
                             0, X, (int)m2, 2 * mm, 0, 0.0, G1 + 2 * mm, (int)m2, 2 * mm, 0,
                             nR - 1);
      gemm_batched<double>(st, false, false, m, (int)m2, m, 1.0, dp(P.SiP), m, 2 * mm, 0, X,
                           (int)m2, 2 * mm, 0, 0.0, G2, (int)m2, 2 * mm, 0, nR);
    } else {
      // Schur products on the tensor cores (split-BF16x3, float32 accumulation)
      unsigned int* err = reinterpret_cast<unsigned int*>(h.info.as<int>()) + 1;
      for (int j = 1; j < nR; ++j)
        tc_gemm_split3(st, m, (int)m2, m, 1.0, dp(P.SiM) + 2 * j * mm, m, X + 2 * (j - 1) * mm,
                       (int)m2, 0.0, G1 + 2 * j * mm, (int)m2, tcws.p, err);
      for (int j = 0; j < nR; ++j)
        tc_gemm_split3(st, m, (int)m2, m, 1.0, dp(P.SiP) + 2 * j * mm, m, X + 2 * j * mm,
                       (int)m2, 0.0, G2 + 2 * j * mm, (int)m2, tcws.p, err);
    }
    if (cyclic) {
      // block 0's left neighbour is the last odd block (index 2 nR - 1)
      gemm_batched<double>(st, false, false, m, (int)m2, m, 1.0, dp(P.SiM), m, 0, 0,
                           X + 2 * (size_t)(nR - 1) * mm, (int)m2, 0, 0, 0.0, G1, (int)m2, 0, 0,
                           1);
    } else {
      SLU_CHECK_CUDA(cudaMemsetAsync(G1, 0, 8 * 2 * mm, st));
    }
    // A = -G1[:, :m]; C = -G2[:, m:]; B = T_even - G1[:, m:] - G2[:, :m]
    copy_batched<double>(st, m, m, dp(P.T), m, 2 * mm, 0, dp(N.T), m, mm, 0, nR);
    add_batched<double>(st, m, m, -1.0, G1 + m, (int)m2, 2 * mm, 0, dp(N.T), m, mm, 0, nR);
    add_batched<double>(st, m, m, -1.0, G2, (int)m2, 2 * mm, 0, dp(N.T), m, mm, 0, nR);
    SLU_CHECK_CUDA(cudaMemsetAsync(dp(N.SiM), 0, 8 * nR * mm, st));
    SLU_CHECK_CUDA(cudaMemsetAsync(dp(N.SiP), 0, 8 * nR * mm, st));
    add_batched<double>(st, m, m, -1.0, G1, (int)m2, 2 * mm, 0, dp(N.SiM), m, mm, 0, nR);
    add_batched<double>(st, m, m, -1.0, G2 + m, (int)m2, 2 * mm, 0, dp(N.SiP), m, mm, 0, nR);
    if (cyclic && nR == 1) {
      // one periodic block: its couplings act on itself (omsdirectsolve.py:326-327)
      add_batched<double>(st, m, m, 1.0, dp(N.SiM), m, 0, 0, dp(N.T), m, 0, 0, 1);
      add_batched<double>(st, m, m, 1.0, dp(N.SiP), m, 0, 0, dp(N.T), m, 0, 0, 1);
    }
    SLU_CHECK_CUDA(cudaMemcpyAsync(dp(N.LU), dp(N.T), 8 * nR * mm, cudaMemcpyDeviceToDevice, st));
    lu_factor(st, m, dp(N.LU), m, mm, ip(N.piv), m, nR, h.info.as<int>());
    make_inverses(st, m, N.LU, N.piv, nR, N.Inv);
    S.levels.push_back(std::move(N));
    l = nR;
  }
  S.fused = false;
  if (m <= kRbFusedMax && !cyclic) build_fused_ops(st, S);
}

void rb_solve(Handle& h, const RbSolver& S, double* B, int ldb, int c, bool tc) {
  if (S.fused && !tc) {
    rb_solve_fused(h, S, B, ldb, c);
    return;
  }
  cudaStream_t st = h.stream;
  const int m = S.m, nblk = S.nblk;
  const size_t mm = (size_t)m * m, mc = (size_t)m * c;
  const int nL = (int)S.levels.size();
  // v[l]: nS_l * m x c
  size_t tot = 0;
  for (const RbLevel& L : S.levels) tot += (size_t)L.nS * mc;
  const size_t tcb = tc ? tc_gemm_workspace_bytes(m, c, m) : 0;
  h.ws.reserve(8 * (tot + (size_t)nblk / 2 * mc + mc) + tcb + 8 * 256, st);
  std::vector<double*> v(nL);
  for (int l = 0; l < nL; ++l) v[l] = h.ws.take<double>((size_t)S.levels[l].nS * mc);
  double* z = h.ws.take<double>(std::max<size_t>(1, (size_t)nblk / 2) * mc);
  void* tcws = tc ? h.ws.take<char>(tcb) : nullptr;
  unsigned int* err = reinterpret_cast<unsigned int*>(h.info.as<int>()) + 1;
  // C_b = alpha A_b V_b + beta C_b for b < batch (A_b m x m, V_b and C_b m x c):
  // float64 batched GEMM, or with `tc` split-BF16x3 tensor-core products
  auto G = [&](double alpha, const double* A, long long sA, const double* V, long long sV,
               double beta, double* C, long long sC, int batch) {
    if (!tc) {
      gemm_batched<double>(st, false, false, m, c, m, alpha, A, m, sA, 0, V, c, sV, 0, beta, C, c,
                           sC, 0, batch);
      return;
    }
    for (int b = 0; b < batch; ++b)
      tc_gemm_split3(st, m, c, m, alpha, A + b * sA, m, V + b * sV, c, beta, C + b * sC, c, tcws,
                     err);
  };
  copy_batched<double>(st, nblk * m, c, B, ldb, 0, 0, v[0], c, 0, 0, 1);
  // forward reduction (omsdirectsolve.py:238-258)
  for (int l = 0; l + 1 < nL; ++l) {
    const RbLevel& P = S.levels[l];
    const int nR = P.nS / 2;
    // z_o = T_o^{-1} v_o (odd o)
    G(1.0, dp(P.Inv) + mm, 2 * mm, v[l] + mc, 2 * mc, 0.0, z, mc, nR);
    // v'_j = v_{2j} - SiM_{2j} z_{2j-1} - SiP_{2j} z_{2j+1}
    copy_batched<double>(st, m, c, v[l], c, 2 * mc, 0, v[l + 1], c, mc, 0, nR);
    if (nR > 1) G(-1.0, dp(P.SiM) + 2 * mm, 2 * mm, z, mc, 1.0, v[l + 1] + mc, mc, nR - 1);
    G(-1.0, dp(P.SiP), 2 * mm, z, mc, 1.0, v[l + 1], mc, nR);
    if (S.cyclic)   // v'_0 -= SiM_0 z_{last odd}
      G(-1.0, dp(P.SiM), 0, z + (size_t)(nR - 1) * mc, 0, 1.0, v[l + 1], 0, 1);
  }
  // coarsest block (omsdirectsolve.py:261)
  G(1.0, dp(S.levels[nL - 1].Inv), 0, v[nL - 1], 0, 0.0, z, 0, 1);
  copy_batched<double>(st, m, c, z, c, 0, 0, v[nL - 1], c, 0, 0, 1);
  // back substitution (omsdirectsolve.py:263-277)
  for (int l = nL - 1; l > 0; --l) {
    const RbLevel& P = S.levels[l - 1];
    const int nR = P.nS / 2;
    // odd blocks first use the coarse (even) solution still stored in v[l]
    // g_o = v_o - SiM_o x_{o-1} - SiP_o x_{o+1}
    G(-1.0, dp(P.SiM) + mm, 2 * mm, v[l], mc, 1.0, v[l - 1] + mc, 2 * mc, nR);
    if (nR > 1) G(-1.0, dp(P.SiP) + mm, 2 * mm, v[l] + mc, mc, 1.0, v[l - 1] + mc, 2 * mc, nR - 1);
    if (S.cyclic)   // the last odd block's right neighbour is block 0
      G(-1.0, dp(P.SiP) + (2 * (size_t)nR - 1) * mm, 0, v[l], 0, 1.0,
        v[l - 1] + (2 * (size_t)nR - 1) * mc, 0, 1);
    G(1.0, dp(P.Inv) + mm, 2 * mm, v[l - 1] + mc, 2 * mc, 0.0, z, mc, nR);
    copy_batched<double>(st, m, c, z, c, mc, 0, v[l - 1] + mc, c, 2 * mc, 0, nR);
    copy_batched<double>(st, m, c, v[l], c, mc, 0, v[l - 1], c, 2 * mc, 0, nR);
  }
  copy_batched<double>(st, nblk * m, c, v[0], c, 0, 0, B, ldb, 0, 0, 1);
}

// ---------------------------------------------------------------- apply / refine
void rb_apply(Handle& h, const RbSolver& S, const double* X, int ldx, double* Y, int ldy, int c) {
  cudaStream_t st = h.stream;
  const int m = S.m, n = S.nblk;
  const size_t mm = (size_t)m * m;
  const RbLevel& L0 = S.levels[0];
  const long long bx = (long long)m * ldx, by = (long long)m * ldy;
  // Y_i = T_i X_i + SiM_i X_{i-1} + SiP_i X_{i+1}  (SiM_0 = SiP_{n-1} = 0)
  gemm_batched<double>(st, false, false, m, c, m, 1.0, dp(L0.T), m, mm, 0, X, ldx, bx, 0, 0.0, Y,
                       ldy, by, 0, n);
  if (n > 1) {
    gemm_batched<double>(st, false, false, m, c, m, 1.0, dp(L0.SiM) + mm, m, mm, 0, X, ldx, bx, 0,
                         1.0, Y + by, ldy, by, 0, n - 1);
    gemm_batched<double>(st, false, false, m, c, m, 1.0, dp(L0.SiP), m, mm, 0, X + bx, ldx, bx, 0,
                         1.0, Y, ldy, by, 0, n - 1);
  }
  if (S.cyclic) {   // wrap-around couplings of a periodic system
    gemm_batched<double>(st, false, false, m, c, m, 1.0, dp(L0.SiM), m, 0, 0,
                         X + (long long)(n - 1) * bx, ldx, 0, 0, 1.0, Y, ldy, 0, 0, 1);
    gemm_batched<double>(st, false, false, m, c, m, 1.0, dp(L0.SiP) + (size_t)(n - 1) * mm, m, 0,
                         0, X, ldx, 0, 0, 1.0, Y + (long long)(n - 1) * by, ldy, 0, 0, 1);
  }
}

namespace {
__global__ void colnorm2_rb(int rows, int cols, const double* __restrict__ A, int lda,
                            double* __restrict__ out) {
  const int c = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    double v = A[(long long)i * lda + c];
    s += v * v;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    out[c] = t;
  }
}
}  // namespace

void rb_refine(Handle& h, const RbSolver& S, const double* B, int ldb, double* X, int ldx, int c,
               double tol, int maxit, int* iters, double* relres) {
  cudaStream_t st = h.stream;
  const int N = S.m * S.nblk;
  DevBuf rb, db, nb;
  rb.alloc(8 * (size_t)N * c, st);
  db.alloc(8 * (size_t)N * c, st);
  nb.alloc(8 * 2 * (size_t)c, st);
  double* r = rb.as<double>();
  double* d = db.as<double>();
  double* bn = nb.as<double>();
  double* rn = bn + c;
  colnorm2_rb<<<c, 256, 0, st>>>(N, c, B, ldb, bn);
  check_launch("colnorm2_rb");
  std::vector<double> hb(c), hr(c);
  SLU_CHECK_CUDA(cudaMemcpyAsync(hb.data(), bn, 8 * c, cudaMemcpyDeviceToHost, st));
  // x0 = A~^{-1} b
  copy_batched<double>(st, N, c, B, ldb, 0, 0, X, ldx, 0, 0, 1);
  rb_solve(h, S, X, ldx, c);
  int it = 1;
  double worst = 0.0;
  for (;;) {
    rb_apply(h, S, X, ldx, r, c, c);                 // r = A x
    add_batched<double>(st, N, c, -1.0, B, ldb, 0, 0, r, c, 0, 0, 1);   // r = A x - b
    colnorm2_rb<<<c, 256, 0, st>>>(N, c, r, c, rn);
    check_launch("colnorm2_rb");
    SLU_CHECK_CUDA(cudaMemcpyAsync(hr.data(), rn, 8 * c, cudaMemcpyDeviceToHost, st));
    stream_wait(st);
    worst = 0.0;
    for (int j = 0; j < c; ++j)
      worst = std::max(worst, std::sqrt(hr[j]) / (hb[j] > 0 ? std::sqrt(hb[j]) : 1.0));
    if (worst <= tol || it >= maxit) break;
    // x -= A~^{-1} (A x - b)
    copy_batched<double>(st, N, c, r, c, 0, 0, d, c, 0, 0, 1);
    rb_solve(h, S, d, c, c);
    add_batched<double>(st, N, c, -1.0, d, c, 0, 0, X, ldx, 0, 0, 1);
    ++it;
  }
  if (iters) *iters = it;
  if (relres) *relres = worst;
  if (worst > tol) throw Error(SLU_ERR_NOT_CONVERGED, "red-black refinement did not reach the tolerance");
}

// ---------------------------------------------------------------- Thomas
void thomas_factor(Handle& h, RbSolver& S, int nblk, int m, const double* SiM, const double* SiP,
                   const double* T) {
  cudaStream_t st = h.stream;
  SLU_REQUIRE(nblk >= 1 && m >= 1, "bad block-tridiagonal geometry");
  S.m = m;
  S.nblk = nblk;
  S.levels.clear();
  S.levels.emplace_back();
  RbLevel& L = S.levels.back();
  const size_t mm = (size_t)m * m;
  L.nS = nblk;
  L.SiM.alloc(8 * nblk * mm, st);  // holds A_i^T = (SiM_i B_{i-1}^{-1})^T (T: A_i)
  L.SiP.alloc(8 * nblk * mm, st);  // C_i
  L.LU.alloc(8 * nblk * mm, st);   // LU(B_i)
  L.piv.alloc(4 * (size_t)nblk * m, st);
  SLU_CHECK_CUDA(cudaMemcpyAsync(dp(L.SiP), SiP, 8 * nblk * mm, cudaMemcpyDeviceToDevice, st));
  SLU_CHECK_CUDA(cudaMemcpyAsync(dp(L.LU), T, 8 * nblk * mm, cudaMemcpyDeviceToDevice, st));
  lu_factor(st, m, dp(L.LU), m, mm, ip(L.piv), m, 1, h.info.as<int>());
  for (int i = 1; i < nblk; ++i) {
    double* At = dp(L.SiM) + i * mm;
    // A_i = SiM_i B_{i-1}^{-1}  ->  A_i^T = B_{i-1}^{-T} SiM_i^T  (omsdirectsolve.py:89-91)
    transpose_batched(st, m, m, SiM + i * mm, m, 0, 0, At, m, 0, 0, 1);
    lu_solve<double>(st, true, m, dp(L.LU) + (i - 1) * mm, m, 0, ip(L.piv) + (i - 1) * m, 0, At,
                     m, 0, m, 1);
    // B_i = T_i - A_i C_{i-1}  (omsdirectsolve.py:94), then LU
    double* Bi = dp(L.LU) + i * mm;
    gemm_batched<double>(st, true, false, m, m, m, -1.0, At, m, 0, 0, dp(L.SiP) + (i - 1) * mm, m,
                         0, 0, 1.0, Bi, m, 0, 0, 1);
    lu_factor(st, m, Bi, m, 0, ip(L.piv) + i * m, 0, 1, h.info.as<int>());
  }
  make_inverses(st, m, L.LU, L.piv, nblk, L.Inv);
  // A_i itself (the solve multiplies by it; block 0 is unused)
  L.T.alloc(8 * nblk * mm, st);
  SLU_CHECK_CUDA(cudaMemsetAsync(dp(L.T), 0, 8 * mm, st));
  if (nblk > 1)
    transpose_batched(st, m, m, dp(L.SiM) + mm, m, (long long)mm, 0, dp(L.T) + mm, m,
                      (long long)mm, 0, nblk - 1);
  S.fused = false;
  if (m <= kRbFusedMax) {
    // fused solve operators (m x 2m per block): Fop_i = [I | -A_i] (i >= 1),
    // Bop_i = [B_i^{-1} | -B_i^{-1} C_i] (the last block: [B^{-1} | 0])
    const long long w = 2LL * m;
    L.Fop.alloc(8 * (size_t)nblk * 2 * mm, st);
    L.Bop.alloc(8 * (size_t)nblk * 2 * mm, st);
    const long long tot = (long long)nblk * 2 * mm;
    ident_wide_kernel<<<(int)std::min<long long>((tot + 255) / 256, 8LL * num_sms()), 256, 0,
                        st>>>(nblk, m, (int)w, dp(L.Fop));
    check_launch("ident_wide_kernel");
    if (nblk > 1)
      add_batched<double>(st, m, m, -1.0, dp(L.T) + mm, m, (long long)mm, 0,
                          dp(L.Fop) + 2 * mm + m, (int)w, 2 * (long long)mm, 0, nblk - 1);
    SLU_CHECK_CUDA(cudaMemsetAsync(dp(L.Bop), 0, 8 * (size_t)nblk * 2 * mm, st));
    copy_batched<double>(st, m, m, dp(L.Inv), m, (long long)mm, 0, dp(L.Bop), (int)w,
                         2 * (long long)mm, 0, nblk);
    if (nblk > 1)
      gemm_batched<double>(st, false, false, m, m, m, -1.0, dp(L.Inv), m, (long long)mm, 0,
                           dp(L.SiP), m, (long long)mm, 0, 0.0, dp(L.Bop) + m, (int)w,
                           2 * (long long)mm, 0, nblk - 1);
    S.fused = true;
  }
}

void thomas_solve(Handle& h, const RbSolver& S, double* B, int ldb, int c) {
  cudaStream_t st = h.stream;
  const int m = S.m, n = S.nblk;
  const size_t mm = (size_t)m * m;
  const RbLevel& L = S.levels[0];
  if (S.fused) {
    // one step kernel per block and sweep: y_i = [I | -A_i] [b_i; y_{i-1}]
    // into Y (y_0 = b_0 copied), then x_i = Bop_i [y_i; x_{i+1}] into B
    // (the last block reads y_{n-1} twice; Bop's right half is zero there)
    const long long mc = (long long)m * c;
    h.ws.reserve(8 * (size_t)n * mc + 256, st);
    double* Y = h.ws.take<double>((size_t)n * mc);
    copy_batched<double>(st, m, c, B, ldb, 0, 0, Y, c, 0, 0, 1);
    auto step = [&](const double* op, const double* in0, int ld0, const double* in1, int ld1,
                    double* out, int ldo) {
      sweep::Step<double> s{};
      s.S = op;
      s.rows = m;
      s.w = 2 * m;
      s.nb = 1;
      s.c = c;
      s.nin = 2;
      s.in_p[0] = in0;
      s.in_ld[0] = ld0;
      s.in_rows[0] = m;
      s.in_p[1] = in1;
      s.in_ld[1] = ld1;
      s.in_rows[1] = m;
      s.split = m;
      s.out_p[0] = out;
      s.out_ld[0] = ldo;
      return s;
    };
    for (int i = 1; i < n; ++i)
      sweep::launch_step(st, step(dp(L.Fop) + 2 * i * mm, B + (size_t)i * m * ldb, ldb,
                                  Y + (i - 1) * mc, c, Y + i * mc, c),
                         "thomas_fwd_step");
    sweep::launch_step(st, step(dp(L.Bop) + 2 * (n - 1) * mm, Y + (n - 1) * mc, c,
                                Y + (n - 1) * mc, c, B + (size_t)(n - 1) * m * ldb, ldb),
                       "thomas_bwd_step");
    for (int i = n - 2; i >= 0; --i)
      sweep::launch_step(st, step(dp(L.Bop) + 2 * i * mm, Y + i * mc, c,
                                  B + (size_t)(i + 1) * m * ldb, ldb, B + (size_t)i * m * ldb,
                                  ldb),
                         "thomas_bwd_step");
    return;
  }
  // d_i -= A_i d_{i-1}  (omsdirectsolve.py:125-126)
  for (int i = 1; i < n; ++i)
    gemm_batched<double>(st, false, false, m, c, m, -1.0, dp(L.T) + i * mm, m, 0, 0,
                         B + (size_t)(i - 1) * m * ldb, ldb, 0, 0, 1.0, B + (size_t)i * m * ldb,
                         ldb, 0, 0, 1);
  // x_n = B_n^{-1} d_n; x_i = B_i^{-1}(d_i - C_i x_{i+1})  (131-139)
  h.ws.reserve(8 * (size_t)m * c + 256, st);
  double* z = h.ws.take<double>((size_t)m * c);
  auto block_solve = [&](int i) {
    double* Bi = B + (size_t)i * m * ldb;
    gemm_batched<double>(st, false, false, m, c, m, 1.0, dp(L.Inv) + i * mm, m, 0, 0, Bi, ldb, 0,
                         0, 0.0, z, c, 0, 0, 1);
    copy_batched<double>(st, m, c, z, c, 0, 0, Bi, ldb, 0, 0, 1);
  };
  block_solve(n - 1);
  for (int i = n - 2; i >= 0; --i) {
    gemm_batched<double>(st, false, false, m, c, m, -1.0, dp(L.SiP) + i * mm, m, 0, 0,
                         B + (size_t)(i + 1) * m * ldb, ldb, 0, 0, 1.0, B + (size_t)i * m * ldb,
                         ldb, 0, 0, 1);
    block_solve(i);
  }
}

}  // namespace slu
