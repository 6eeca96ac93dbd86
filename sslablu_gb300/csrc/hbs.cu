// HBS compression, ULV factorisation, apply and solve drivers.
//
// Follows the level recursions of
//   matAssembly/HBS/HBSnew.py:211-295  (constructHBS_ULV: compression leaf ->
//                                       root with the ULV interleaved)
//   matAssembly/HBS/HBSnew.py:308-350  (matmat / rmatmat)
//   matAssembly/HBS/HBSnew.py:393-416  (solve with the tree permutation)
//   matAssembly/HBS/ULVsparse.py:64-100, 231-358 (compute_QRW_sparse,
//                                       compute_ULV, solve N/T)
// with every per-block loop replaced by one batched launch per level.
//
// Right pseudo-inverses X * pinv(Om_blk) (HBSnew.py:11-19, 48-62) are
// evaluated as X * Q_1 * R^{-T} from the Householder QR Om_blk^T = Q_1 R that
// compute_UV already needs, so each sketch block is factored once.  For the
// full-row-rank Gaussian sketches this equals upstream's SVD pseudo-inverse
// (rcond 1e-15 never truncates) to rounding.
#include "hbs.cuh"

#include <algorithm>
#include <utility>

namespace slu {
namespace {

inline double* dp(const DevBuf& b) { return b.as<double>(); }

template <typename T>
inline void gemm(cudaStream_t st, bool ta, bool tb, int M, int N, int K, T alpha, const T* A,
                 int lda, long long sA0, long long sA1, const T* B, int ldb, long long sB0,
                 long long sB1, T beta, T* C, int ldc, long long sC0, long long sC1, int b0,
                 int b1 = 1) {
  gemm_batched<T>(st, ta, tb, M, N, K, alpha, A, lda, sA0, sA1, B, ldb, sB0, sB1, beta, C, ldc,
                  sC0, sC1, b0, b1);
}

inline void alloc_d(DevBuf& b, size_t count, cudaStream_t st) { b.alloc(count * sizeof(double), st); }

void setup_geometry_common(Hbs& H) {
  H.NN.assign(H.L + 1, 0);
  for (int t = 0; t < H.L; ++t) {
    Level& l = H.lv[t];
    const bool root = (t == H.L - 1);
    l.nu = root ? l.n : l.n - l.k;
    H.NN[t + 1] = H.NN[t] + (long long)l.nu * l.Nb;
  }
}

// ---------------------------------------------------------------- ULV level
// One level of ULVsparse.compute_QRW_sparse (ULVsparse.py:64-100) plus the
// Uhat recursion of compute_ULV / constructHBS_ULV (ULVsparse.py:273-287,
// HBSnew.py:273-294).
//   Rhat      : Nb*n x n (leaf: D; above: blkdiag(Ud_children) D + blkdiag(R22))
//   Uhat      : Nb*n x kU
//   kslice    : split of Q^T Uhat into Uu (first n-kslice rows) and Ud
//   Ud_out    : Nb*kslice x kU, R22_out: Nb*k x k (non-root)
struct UlvScratch {
  double *WSV, *tauV, *Qk, *DWt, *tauQ, *Qc, *QtU;
};

void ulv_level(cudaStream_t st, Level& l, bool root, const double* Rhat, const double* Uhat,
               int kU, int kslice, bool store_uu, double* Ud_out, double* R22_out,
               const UlvScratch& s) {
  const int Nb = l.Nb, n = l.n, k = root ? 0 : l.k, nu = l.nu;
  const long long nn = (long long)n * n;
  if (!root) {
    // W1: trailing n-k columns of the complete QR of each V block (ULVsparse.py:18-25)
    transpose_batched(st, n, k, dp(l.V), k, (long long)n * k, 0, s.WSV, n, (long long)n * k, 0, Nb);
    panel_qr(st, n, k, k, s.WSV, n, (long long)n * k, s.tauV, k, Nb);
    if (n > k) {
      identity_cols(st, n, k, n - k, s.Qk, (long long)n * (n - k), Nb);
      apply_q(st, false, n, k, s.WSV, n, (long long)n * k, s.tauV, k, s.Qk, n,
              (long long)n * (n - k), n - k, Nb);
      // W = [W1 | V]  (row-major n x n)
      transpose_batched(st, n - k, n, s.Qk, n, (long long)n * (n - k), 0, dp(l.W), n, nn, 0, Nb);
    }
    copy_batched<double>(st, n, k, dp(l.V), k, (long long)n * k, 0, dp(l.W) + (n - k), n, nn, 0,
                         Nb);
    // (Rhat W)^T = W^T Rhat^T: row-major result == column-major Rhat W
    gemm<double>(st, true, true, n, n, n, 1.0, dp(l.W), n, nn, 0, Rhat, n, nn, 0, 0.0, s.DWt, n,
                 nn, 0, Nb);
  } else {
    transpose_batched(st, n, n, Rhat, n, nn, 0, s.DWt, n, nn, 0, Nb);
  }
  // square QR of Rhat W (ULVsparse.py:51-61)
  panel_qr(st, n, n, n, s.DWt, n, nn, s.tauQ, n, Nb);
  extract_upper(st, 0, nu, 0, n, s.DWt, n, nn, dp(l.R), n, (long long)nu * n, Nb);
  if (!root && k > 0) extract_upper(st, nu, k, nu, k, s.DWt, n, nn, R22_out, k, (long long)k * k, Nb);
  identity_cols(st, n, 0, n, s.Qc, nn, Nb);
  apply_q(st, false, n, n, s.DWt, n, nn, s.tauQ, n, s.Qc, n, nn, n, Nb);
  transpose_batched(st, n, n, s.Qc, n, nn, 0, dp(l.Q), n, nn, 0, Nb);
  // Q^T Uhat -> Uu (leading rows) and Ud (trailing kslice rows)
  if (kU > 0 && (store_uu || !root)) {
    gemm<double>(st, true, false, n, kU, n, 1.0, dp(l.Q), n, nn, 0, Uhat, kU, (long long)n * kU,
                 0, 0.0, s.QtU, kU, (long long)n * kU, 0, Nb);
    if (store_uu && n > kslice)
      copy_blocks(st, Nb, (long long)(n - kslice) * kU * 8, s.QtU, (long long)n * kU * 8,
                  dp(l.Uu), (long long)(n - kslice) * kU * 8);
    if (!root)
      copy_blocks(st, Nb, (long long)kslice * kU * 8, s.QtU + (long long)(n - kslice) * kU,
                  (long long)n * kU * 8, Ud_out, (long long)kslice * kU * 8);
  }
}

size_t ulv_scratch_doubles(const Hbs& H) {
  size_t m = 0;
  for (const Level& l : H.lv) {
    size_t nb = l.Nb, n = l.n, k = l.k;
    size_t kU = std::max<size_t>(k, n);
    m = std::max(m, nb * (n * k + k + n * n + n * n + n + n * n + n * kU));
  }
  return m;
}

UlvScratch carve_ulv(Workspace& ws, const Hbs& H) {
  size_t a = 0, b = 0, c = 0, d = 0, e = 0;
  for (const Level& l : H.lv) {
    size_t nb = l.Nb, n = l.n, k = l.k;
    a = std::max(a, nb * n * std::max<size_t>(k, 1));
    b = std::max(b, nb * std::max<size_t>(k, 1));
    c = std::max(c, nb * n * n);
    d = std::max(d, nb * n);
    e = std::max(e, nb * n * std::max<size_t>(std::max<size_t>(k, n), 1));
  }
  UlvScratch s;
  s.WSV = ws.take<double>(a);
  s.tauV = ws.take<double>(b);
  s.Qk = ws.take<double>(c);
  s.DWt = ws.take<double>(c);
  s.tauQ = ws.take<double>(d);
  s.Qc = ws.take<double>(c);
  s.QtU = ws.take<double>(e);
  return s;
}

size_t ulv_scratch_bytes(const Hbs& H) {
  size_t a = 0, b = 0, c = 0, d = 0, e = 0;
  for (const Level& l : H.lv) {
    size_t nb = l.Nb, n = l.n, k = l.k;
    a = std::max(a, nb * n * std::max<size_t>(k, 1));
    b = std::max(b, nb * std::max<size_t>(k, 1));
    c = std::max(c, nb * n * n);
    d = std::max(d, nb * n);
    e = std::max(e, nb * n * std::max<size_t>(std::max<size_t>(k, n), 1));
  }
  return 8 * (a + b + 3 * c + d + e) + 7 * 256;
}

// Rhat / Uhat of a non-leaf level from the children's Ud and R22.
void merge_children(cudaStream_t st, const Hbs& H, int t, const double* Ud_c, const double* R22_c,
                    double* Rhat, double* Uhat, bool root_uhat) {
  const Level& l = H.lv[t];
  const Level& c = H.lv[t - 1];
  const int fac = H.fac, Nb = l.Nb, n = l.n, kc = c.k;
  const long long kk = (long long)kc * kc, nn = (long long)n * n;
  // Rhat = blkdiag(Ud_children) D + blkdiag(R22_children)  (ULVsparse.py:263-264)
  gemm<double>(st, false, false, kc, n, kc, 1.0, Ud_c, kc, kk, fac * kk, dp(l.D), n,
               (long long)kc * n, nn, 0.0, Rhat, n, (long long)kc * n, nn, fac, Nb);
  add_batched<double>(st, kc, kc, 1.0, R22_c, kc, kk, fac * kk, Rhat, n, (long long)kc * n + kc,
                      nn, fac, Nb);
  const bool root = (t == H.L - 1);
  if (!root) {
    // Uhat = blkdiag(Ud_children) U  (ULVsparse.py:283)
    const int k = l.k;
    gemm<double>(st, false, false, kc, k, kc, 1.0, Ud_c, kc, kk, fac * kk, dp(l.U), k,
                 (long long)kc * k, (long long)n * k, 0.0, Uhat, k, (long long)kc * k,
                 (long long)n * k, fac, Nb);
  } else if (root_uhat) {
    // root: U = I, Uhat = blkdiag(Ud_children)  (HBSnew.py:271, 289)
    SLU_CHECK_CUDA(cudaMemsetAsync(Uhat, 0, sizeof(double) * nn, st));
    copy_batched<double>(st, kc, kc, Ud_c, kc, kk, 0, Uhat, n, (long long)kc * n + kc, 0, fac);
  }
}

}  // namespace

// ============================================================== compression
void hbs_compress(Handle& h, Hbs& H, int Nb0, int rk, int s, const double* Om, const double* Psi,
                  const double* Y, const double* Z, bool ulv) {
  cudaStream_t st = h.stream;
  const int N = H.N, L = H.L, fac = H.fac;
  SLU_REQUIRE(L >= 1 && N > 0, "bad HBS geometry");
  long long p = 1;
  for (int t = 1; t < L; ++t) p *= fac;
  SLU_REQUIRE(Nb0 == p, "leaf count must equal fac^(L-1)");
  const int nl = N / Nb0;
  SLU_REQUIRE((long long)nl * Nb0 == N, "N must be a multiple of the leaf count");
  SLU_REQUIRE(rk >= 1, "rank must be positive");
  // ---- level geometry (HBSnew.py:234-256)
  H.lv.clear();
  H.lv.resize(L);
  {
    int Nb = Nb0, n = nl;
    long long nomin = nl;
    for (int t = 0; t < L; ++t) {
      Level& l = H.lv[t];
      l.Nb = Nb;
      l.n = n;
      int rkm = (int)std::min<long long>(rk, nomin);
      l.k = (t < L - 1) ? rkm : 0;
      Nb /= fac;
      n = fac * rkm;
      nomin *= fac;
    }
  }
  setup_geometry_common(H);
  for (int t = 0; t < L; ++t) {
    Level& l = H.lv[t];
    const bool root = (t == L - 1);
    l.kU = root ? l.n : l.k;
    l.uu_rows = root ? std::max(l.n - rk, 0) : l.n - l.k;
    const size_t rows = (size_t)l.Nb * l.n;
    if (!root) {
      alloc_d(l.U, rows * l.k, st);
      alloc_d(l.V, rows * l.k, st);
      if (ulv) alloc_d(l.W, rows * l.n, st);
    }
    alloc_d(l.D, rows * l.n, st);
    if (ulv) {
      alloc_d(l.Q, rows * l.n, st);
      alloc_d(l.R, (size_t)l.Nb * l.nu * l.n, st);
      alloc_d(l.Uu, (size_t)l.Nb * l.uu_rows * l.kU, st);
    }
  }
  H.rk = rk;
  H.nsamples = s;
  // ---- workspace
  size_t Ns = (size_t)N * s;
  size_t nmax = 0, kmax = 1;
  for (const Level& l : H.lv) { nmax = std::max<size_t>(nmax, l.n); kmax = std::max<size_t>(kmax, l.k); }
  size_t need = 8 * (8 * Ns + 4 * Ns + 2 * (size_t)N + 3 * (size_t)N * nmax) + 32 * 256;
  if (ulv) need += ulv_scratch_bytes(H) + 8 * (2 * (size_t)N * nmax + 4 * (size_t)N * kmax) + 8 * 256;
  h.ws.reserve(need, st);
  double* set[2][4];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 4; ++b) set[a][b] = h.ws.take<double>(Ns);
  double* WSA = h.ws.take<double>(2 * Ns);
  double* WSB = h.ws.take<double>(2 * Ns);
  double* tauA = h.ws.take<double>(N);
  double* tauB = h.ws.take<double>(N);
  double* PB = h.ws.take<double>((size_t)N * nmax);
  double* T1 = h.ws.take<double>((size_t)N * nmax);
  double* T2 = h.ws.take<double>((size_t)N * nmax);
  UlvScratch us{};
  double *Rhat = nullptr, *Uhat = nullptr, *Ud[2] = {nullptr, nullptr}, *R22[2] = {nullptr, nullptr};
  if (ulv) {
    us = carve_ulv(h.ws, H);
    Rhat = h.ws.take<double>((size_t)N * nmax);
    Uhat = h.ws.take<double>((size_t)N * nmax);
    for (int a = 0; a < 2; ++a) {
      Ud[a] = h.ws.take<double>((size_t)N * kmax);
      R22[a] = h.ws.take<double>((size_t)N * kmax);
    }
  }
  // leaf sketches: Om/Psi read in place, Y/Z copied (they are updated in place)
  const double* Om_t = Om;
  const double* Psi_t = Psi;
  double* Y_t = set[0][2];
  double* Z_t = set[0][3];
  SLU_CHECK_CUDA(cudaMemcpyAsync(Y_t, Y, 8 * Ns, cudaMemcpyDeviceToDevice, st));
  SLU_CHECK_CUDA(cudaMemcpyAsync(Z_t, Z, 8 * Ns, cudaMemcpyDeviceToDevice, st));
  int cur = 0;
  for (int t = 0; t < L; ++t) {
    Level& l = H.lv[t];
    const bool root = (t == L - 1);
    const int Nb = l.Nb, n = l.n, k = l.k;
    const long long ns = (long long)n * s, nn = (long long)n * n;
    if (t > 0) {
      // sketch update from the child level (HBSnew.py:244-251)
      const Level& c = H.lv[t - 1];
      const int nc = c.n, kc = c.k, Nbc = c.Nb;
      const long long ncs = (long long)nc * s, kcs = (long long)kc * s, ncc = (long long)nc * nc;
      const int nxt = cur ^ 1;
      double* Om_n = set[nxt][0];
      double* Psi_n = set[nxt][1];
      double* Y_n = set[nxt][2];
      double* Z_n = set[nxt][3];
      gemm<double>(st, false, false, nc, s, nc, -1.0, dp(c.D), nc, ncc, 0, Om_t, s, ncs, 0, 1.0,
                   Y_t, s, ncs, 0, Nbc);
      gemm<double>(st, true, false, kc, s, nc, 1.0, dp(c.U), kc, (long long)nc * kc, 0, Y_t, s,
                   ncs, 0, 0.0, Y_n, s, kcs, 0, Nbc);
      gemm<double>(st, true, false, nc, s, nc, -1.0, dp(c.D), nc, ncc, 0, Psi_t, s, ncs, 0, 1.0,
                   Z_t, s, ncs, 0, Nbc);
      gemm<double>(st, true, false, kc, s, nc, 1.0, dp(c.V), kc, (long long)nc * kc, 0, Z_t, s,
                   ncs, 0, 0.0, Z_n, s, kcs, 0, Nbc);
      gemm<double>(st, true, false, kc, s, nc, 1.0, dp(c.V), kc, (long long)nc * kc, 0, Om_t, s,
                   ncs, 0, 0.0, Om_n, s, kcs, 0, Nbc);
      gemm<double>(st, true, false, kc, s, nc, 1.0, dp(c.U), kc, (long long)nc * kc, 0, Psi_t, s,
                   ncs, 0, 0.0, Psi_n, s, kcs, 0, Nbc);
      Om_t = Om_n;
      Psi_t = Psi_n;
      Y_t = Y_n;
      Z_t = Z_n;
      cur = nxt;
    }
    // ---- side A: QR of Om_blk^T with Y_blk rows carried along (compute_UV)
    // (sides A and B run as one launch each: independent problems of the
    // same shapes, so a level with few blocks fills twice as many SMs)
    copy_blocks(st, Nb, 8 * ns, Om_t, 8 * ns, WSA, 16 * ns);
    copy_blocks(st, Nb, 8 * ns, Y_t, 8 * ns, WSA + ns, 16 * ns);
    if (root) panel_qr(st, s, n, 2 * n, WSA, s, 2 * ns, tauA, n, Nb);
    const double* YQ1A = WSA + ns;   // row-major n x n (ld s): Y_blk * Q_1
    if (!root) {
      copy_blocks(st, Nb, 8 * ns, Psi_t, 8 * ns, WSB, 16 * ns);
      copy_blocks(st, Nb, 8 * ns, Z_t, 8 * ns, WSB + ns, 16 * ns);
      panel_qr2(st, s, n, 2 * n, WSA, WSB, s, 2 * ns, tauA, tauB, n, Nb);
      int* info = h.info.as<int>();
      // U, V: leading left singular vectors of Y_blk Q[:, s-n:s] (HBSnew.py:26-27)
      // or of Y_blk Q[:, n:s] (HBStorch.py:73-82)
      const int jc = H.null_after_n ? s - n : n;
      const int j0 = H.null_after_n ? n : s - n;
      SLU_REQUIRE(k <= std::min(n, jc), "rank exceeds the columns of the projected sketch");
      if (jc > n) {
        // wide n x jc block: its left singular vectors are those of R^T from
        // the QR of its transpose, which the panels already hold column-major
        // (column i = row i of the block); R^T is n x n lower triangular
        panel_qr2(st, jc, n, n, WSA + ns + j0, WSB + ns + j0, s, 2 * ns, tauA, tauB, n, Nb);
        jacobi_left_sv2(st, n, n, WSA + ns + j0, WSB + ns + j0, s, 2 * ns, k, dp(l.U), dp(l.V),
                        k, (long long)n * k, Nb, info, true);
      } else {
        jacobi_left_sv2(st, n, jc, WSA + ns + j0, WSB + ns + j0, s, 2 * ns, k, dp(l.U), dp(l.V),
                        k, (long long)n * k, Nb, info);
      }
      // D = (Y - U U^T Y) pinv(Om) + U U^T ((Z - V V^T Z) pinv(Psi))^T  (HBSnew.py:48-62)
      const long long nk = (long long)n * k;
      copy_batched<double>(st, n, n, YQ1A, s, 2 * ns, 0, dp(l.D), n, nn, 0, Nb);
      gemm<double>(st, true, false, k, n, n, 1.0, dp(l.U), k, nk, 0, YQ1A, s, 2 * ns, 0, 0.0, T1,
                   n, nk, 0, Nb);
      gemm<double>(st, false, false, n, n, k, -1.0, dp(l.U), k, nk, 0, T1, n, nk, 0, 1.0, dp(l.D),
                   n, nn, 0, Nb);
      trsm_upper<double>(st, false, n, WSA, 1, s, 2 * ns, dp(l.D), 1, n, nn, n, Nb);
      const double* YQ1B = WSB + ns;
      copy_batched<double>(st, n, n, YQ1B, s, 2 * ns, 0, PB, n, nn, 0, Nb);
      gemm<double>(st, true, false, k, n, n, 1.0, dp(l.V), k, nk, 0, YQ1B, s, 2 * ns, 0, 0.0, T1,
                   n, nk, 0, Nb);
      gemm<double>(st, false, false, n, n, k, -1.0, dp(l.V), k, nk, 0, T1, n, nk, 0, 1.0, PB, n,
                   nn, 0, Nb);
      trsm_upper<double>(st, false, n, WSB, 1, s, 2 * ns, PB, 1, n, nn, n, Nb);
      gemm<double>(st, true, true, k, n, n, 1.0, dp(l.U), k, nk, 0, PB, n, nn, 0, 0.0, T2, n, nk,
                   0, Nb);
      gemm<double>(st, false, false, n, n, k, 1.0, dp(l.U), k, nk, 0, T2, n, nk, 0, 1.0, dp(l.D),
                   n, nn, 0, Nb);
    } else {
      // root: D = Y pinv(Om)  (HBSnew.py:11-19, 268)
      copy_batched<double>(st, n, n, YQ1A, s, 2 * ns, 0, dp(l.D), n, nn, 0, Nb);
      trsm_upper<double>(st, false, n, WSA, 1, s, 2 * ns, dp(l.D), 1, n, nn, n, Nb);
    }
    // ---- interleaved ULV (HBSnew.py:273-294)
    if (ulv) {
      const int w = t & 1, r = w ^ 1;  // write / read slots of Ud, R22
      const double* Rh = dp(l.D);
      const double* Uh = root ? Uhat : dp(l.U);
      if (t == 0 && root) identity_cols(st, n, 0, n, Uhat, nn, 1);  // single-level tree: U = I
      if (t > 0) {
        merge_children(st, H, t, Ud[r], R22[r], Rhat, Uhat, true);
        Rh = Rhat;
        Uh = Uhat;
      }
      // upstream slices Q[:, :-rk] / Q[:, -rk:] (HBSnew.py:291-292); Python
      // slicing saturates, so the split is min(rk, n) = the level rank below
      // the root
      const int kslice = root ? std::min(rk, n) : l.k;
      ulv_level(st, l, root, Rh, Uh, l.kU, kslice, true, Ud[w], R22[w], us);
    }
  }
  H.has_mats = true;
  H.has_ulv = ulv;
  H.has_f32 = false;
  H.has_dfs = false;
  H.has_df = false;
  H.has_sweep = false;
  H.has_oz = H.has_ozT = false;
  H.has_apply[0] = H.has_apply[1] = false;
  H.invalidate_plans();
  if (ulv) hbs_make_sweep(h, H);
}

// ============================================================== standalone ULV
void hbs_factor(Handle& h, Hbs& H) {
  cudaStream_t st = h.stream;
  SLU_REQUIRE(H.has_mats, "HBS factors not loaded");
  for (int t = 0; t + 1 < H.L; ++t)
    SLU_REQUIRE(H.lv[t].V.p, "factorisation needs V factors (loaded without V)");
  const int L = H.L;
  size_t nmax = 0, kmax = 1, N = H.N;
  for (const Level& l : H.lv) { nmax = std::max<size_t>(nmax, l.n); kmax = std::max<size_t>(kmax, l.k); }
  for (int t = 0; t < L; ++t) {
    Level& l = H.lv[t];
    const bool root = (t == L - 1);
    l.kU = root ? 0 : l.k;
    l.uu_rows = root ? 0 : l.n - l.k;
    const size_t rows = (size_t)l.Nb * l.n;
    if (!root) alloc_d(l.W, rows * l.n, st);
    alloc_d(l.Q, rows * l.n, st);
    alloc_d(l.R, (size_t)l.Nb * l.nu * l.n, st);
    if (!root) alloc_d(l.Uu, (size_t)l.Nb * l.uu_rows * l.kU, st);
  }
  h.ws.reserve(ulv_scratch_bytes(H) + 8 * (2 * N * nmax + 4 * N * kmax) + 8 * 256, st);
  UlvScratch us = carve_ulv(h.ws, H);
  double* Rhat = h.ws.take<double>(N * nmax);
  double* Uhat = h.ws.take<double>(N * nmax);
  double *Ud[2], *R22[2];
  for (int a = 0; a < 2; ++a) {
    Ud[a] = h.ws.take<double>(N * kmax);
    R22[a] = h.ws.take<double>(N * kmax);
  }
  for (int t = 0; t < L; ++t) {
    Level& l = H.lv[t];
    const bool root = (t == L - 1);
    const int w = t & 1, r = w ^ 1;
    const double* Rh = dp(l.D);
    const double* Uh = root ? nullptr : dp(l.U);
    if (t > 0) {
      merge_children(st, H, t, Ud[r], R22[r], Rhat, Uhat, false);
      Rh = Rhat;
      Uh = Uhat;
    }
    ulv_level(st, l, root, Rh, Uh, l.kU, l.k, !root, Ud[w], R22[w], us);
  }
  H.has_ulv = true;
  H.has_f32 = false;
  H.has_dfs = false;
  H.has_oz = H.has_ozT = false;   // digit forms of the step operators are stale
  H.invalidate_plans();
  hbs_make_sweep(h, H);
}

// ============================================================== apply
void hbs_apply(Handle& h, Hbs& H, bool trans, const double* X, int ldx, double* Yout,
               int ldy, int c) {
  cudaStream_t st = h.stream;
  SLU_REQUIRE(H.has_mats, "HBS factors not loaded");
  if (!H.has_apply[trans ? 1 : 0]) {
    std::lock_guard<std::mutex> lock(H.lazy_mu);
    if (!H.has_apply[trans ? 1 : 0]) hbs_make_apply(h, H, trans);
  }
  const size_t elems = hbs_apply_scratch_elems(H, c);
  h.ws.reserve(8 * elems + 256, st);
  double* scratch = h.ws.take<double>(elems);
  hbs_apply_fused<double>(st, H, trans, X, ldx, Yout, ldy, c, scratch);
}

// ============================================================== solve
size_t hbs_solve_scratch_bytes(const Hbs& H, int c, size_t elem) {
  return 5 * ((elem * (size_t)H.N * c + 255) & ~size_t(255));
}

template <typename T>
void hbs_solve(Handle& h, const Hbs& H, bool trans, T* B, int ldb, int c) {
  h.ws.reserve(hbs_solve_scratch_bytes(H, c, sizeof(T)) + 256, h.stream);
  T* scratch = h.ws.take<T>(hbs_solve_scratch_bytes(H, c, sizeof(T)) / sizeof(T));
  hbs_solve_scratch<T>(h.stream, H, trans, B, ldb, c, scratch);
}

template <typename T>
void hbs_solve_scratch(cudaStream_t st, const Hbs& H, bool trans, T* B, int ldb, int c,
                       T* scratch) {
  SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
  if (sizeof(T) == 4) SLU_REQUIRE(H.has_f32, "single-precision factors not prepared");
  // five (N x c) buffers, each starting on a 256-byte boundary
  const size_t stride = ((sizeof(T) * (size_t)H.N * c + 255) & ~size_t(255)) / sizeof(T);
  if (!trans) {
    // mode N (ULVsparse.py:296-327): one step kernel per tree step
    ulv_solve_fused<T>(st, H, B, ldb, c, scratch, stride);
  } else {
    // mode T (ULVsparse.py:328-353): the transposed steps, in reverse order;
    // upstream scatters the input and gathers the output (HBSnew.py:403-411)
    ulv_solve_T<T>(st, H, B, ldb, c, scratch, stride);
  }
}
template void hbs_solve<double>(Handle&, const Hbs&, bool, double*, int, int);
template void hbs_solve<float>(Handle&, const Hbs&, bool, float*, int, int);
template void hbs_solve_scratch<double>(cudaStream_t, const Hbs&, bool, double*, int, int, double*);
template void hbs_solve_scratch<float>(cudaStream_t, const Hbs&, bool, float*, int, int, float*);

void hbs_make_f32(Handle& h, Hbs& H) {
  cudaStream_t st = h.stream;
  H.invalidate_plans();
  SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
  auto cp = [&](const DevBuf& src, DevBuf& dst) {
    size_t n = src.bytes / 8;
    dst.alloc(n * 4, st);
    cast_f64_f32(st, (long long)n, src.as<double>(), dst.as<float>());
  };
  SLU_REQUIRE(H.has_sweep, "step operators not composed");
  for (Level& l : H.lv) {
    cp(l.U, l.Uf);
    cp(l.D, l.Df);
    cp(l.Q, l.Qf);
    cp(l.W, l.Wf);
    cp(l.R, l.Rf);
    cp(l.Uu, l.Uuf);
    cp(l.Qt, l.Qtf);
    cp(l.Sw, l.Swf);
    cp(l.SwT, l.SwTf);
  }
  if (H.top >= 1) cp(H.Top, H.Topf);
  H.has_f32 = true;
}

size_t hbs_nbytes(const Hbs& H, int which) {
  size_t b = 0;
  for (const Level& l : H.lv) {
    if (which == 0) b += l.U.bytes + l.V.bytes + l.D.bytes;
    else b += l.U.bytes + l.D.bytes + l.Q.bytes + l.W.bytes + l.R.bytes + l.Uu.bytes;
  }
  return b;
}

}  // namespace slu
