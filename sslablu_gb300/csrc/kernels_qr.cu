// Householder QR panels, reflector application and one-sided Jacobi SVD.
//
// These implement the per-block LAPACK work of the HBS compression and ULV
// factorisation:
//   * complete QR of each sketch block Om_blk^T and the projection of Y onto
//     the trailing columns of Q (matAssembly/HBS/HBSnew.py:20-28 compute_UV),
//     which also yields Y*Q_1 and R for the right pseudo-inverse solves of
//     construct_D / block_solve_r (HBSnew.py:11-19, 48-62);
//   * the SVD whose leading left singular vectors become U (HBSnew.py:27);
//   * complete QR of V (W1, ULVsparse.py:18-25) and square QR of D*W
//     (ULVsparse.py:51-61).
// Reflectors follow the LAPACK geqrf convention (beta = -sign(alpha)*norm,
// v[0] = 1), so the trailing columns of Q match LAPACK's to rounding.
#include <algorithm>

#include "slablu_internal.cuh"

namespace slu {
namespace {

__device__ inline double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ inline double block_sum(double v, double* red) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  double t = 0.0;
  for (int i = 0; i < nw; ++i) t += red[i];
  return t;
}

// QR of the first nfac columns of an m x ncol column-major work array `a`
// (leading dimension lda), applying each reflector to every later column.
__device__ void panel_qr_dev(int m, int nfac, int ncol, double* a, int lda, double* tau) {
  __shared__ double red[32];
  __shared__ double s_tau, s_scale;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int j = 0; j < nfac && j < m; ++j) {
    double* col = a + (long long)j * lda;
    double ss = 0.0;
    for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) ss += col[i] * col[i];
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) {
      double alpha = col[j];
      if (ss == 0.0) {
        s_tau = 0.0;
        s_scale = 0.0;
      } else {
        double beta = -copysign(sqrt(alpha * alpha + ss), alpha);
        s_tau = (beta - alpha) / beta;
        s_scale = 1.0 / (alpha - beta);
        col[j] = beta;
      }
      tau[j] = s_tau;
    }
    __syncthreads();
    const double t = s_tau, sc = s_scale;
    if (t != 0.0)
      for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] *= sc;
    __syncthreads();
    if (t != 0.0) {
      for (int c = j + 1 + warp; c < ncol; c += nwarps) {
        double* cc = a + (long long)c * lda;
        double d = (lane == 0) ? cc[j] : 0.0;
        for (int i = j + 1 + lane; i < m; i += 32) d += col[i] * cc[i];
        d = warp_sum(d) * t;
        if (lane == 0) cc[j] -= d;
        for (int i = j + 1 + lane; i < m; i += 32) cc[i] -= d * col[i];
      }
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(512)
panel_qr_kernel(int m, int nfac, int ncol, double* __restrict__ W, int ldw, long long sW,
                double* __restrict__ tau, long long sTau, int use_smem, double* __restrict__ W2,
                double* __restrict__ tau2, int nsplit) {
  extern __shared__ double sm[];
  // blocks nsplit.. work on the second batch (W2, tau2), same shapes
  const bool second = (int)blockIdx.x >= nsplit;
  const long long b = second ? blockIdx.x - nsplit : blockIdx.x;
  double* w = (second ? W2 : W) + b * sW;
  double* t = (second ? tau2 : tau) + b * sTau;
  if (use_smem) {
    for (long long e = threadIdx.x; e < (long long)m * ncol; e += blockDim.x) {
      int c = (int)(e / m), i = (int)(e % m);
      sm[e] = w[(long long)c * ldw + i];
    }
    __syncthreads();
    panel_qr_dev(m, nfac, ncol, sm, m, t);
    __syncthreads();
    for (long long e = threadIdx.x; e < (long long)m * ncol; e += blockDim.x) {
      int c = (int)(e / m), i = (int)(e % m);
      w[(long long)c * ldw + i] = sm[e];
    }
  } else {
    panel_qr_dev(m, nfac, ncol, w, ldw, t);
  }
}

// C <- Q C (transpose = false) or Q^T C; each warp owns whole columns of C.
__global__ void __launch_bounds__(256)
apply_q_kernel(bool transpose, int m, int k, const double* __restrict__ V, int ldv, long long sV,
               const double* __restrict__ tau, long long sTau, double* __restrict__ C, int ldc,
               long long sC, int nc) {
  V += blockIdx.y * sV;
  tau += blockIdx.y * sTau;
  C += blockIdx.y * sC;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int c = blockIdx.x * nwarps + warp;
  if (c >= nc) return;
  double* cc = C + (long long)c * ldc;
  for (int s = 0; s < k; ++s) {
    const int j = transpose ? s : (k - 1 - s);
    const double t = tau[j];
    if (t == 0.0) continue;
    const double* v = V + (long long)j * ldv;
    double d = (lane == 0) ? cc[j] : 0.0;
    for (int i = j + 1 + lane; i < m; i += 32) d += v[i] * cc[i];
    d = warp_sum(d) * t;
    if (lane == 0) cc[j] -= d;
    for (int i = j + 1 + lane; i < m; i += 32) cc[i] -= d * v[i];
    __syncwarp();
  }
}

// ---------------------------------------------------------------- Jacobi SVD
// One-sided (Hestenes) Jacobi on the columns of A (m x n), round-robin pair
// ordering.  Each column pair belongs to JAC_LANES consecutive lanes of a
// warp; a lane owns rows part, part + JAC_LANES, ...  The lanes form the
// three inner products of the pair over their rows (two partial sums each,
// then a shuffle butterfly -- the pair's sums are combined the same way on
// every lane), compute the rotation redundantly and rotate their own rows,
// so no shared-memory traffic beyond the columns themselves and one block
// barrier per round.  The rotation is orthogonal in float64 whatever its
// angle, so the angle is computed in float32 from the float64 quotient
// zeta = (beta - alpha) / (2 gamma) and the float64 (c, s) are renormalised
// to c^2 + s^2 = 1 to float64 rounding; an angle good to ~1e-7 still cuts
// gamma by that factor per rotation, and the sweep test (|gamma| <= m eps
// sqrt(alpha beta) for every pair) is unchanged.  Small angles
// (|zeta| > 1e7, where zeta^2 would leave float32 range) take t = 1/(2 zeta)
// in float64 instead.  Columns live in shared
// memory with an odd leading dimension.  At convergence the columns are
// sigma_j u_j; the r largest are normalised and written as U (m x r).
constexpr int JAC_MAX_SWEEPS = 40;
constexpr int JAC_LANES = 4;

__global__ void __launch_bounds__(1024)
jacobi_kernel(int m, int n, const double* __restrict__ A, int lda, long long sA, int r,
              double* __restrict__ U, int ldu, long long sU, double* __restrict__ sv,
              long long sS, int* info, int lower, const double* __restrict__ A2,
              double* __restrict__ U2, int nsplit) {
  extern __shared__ double sm[];
  const int np = n + (n & 1);            // even number of columns (a zero pad column)
  const int lda_s = m | 1;               // odd column stride
  double* a = sm;                        // column-major, column c at a + c * lda_s
  double* nrm = a + (long long)lda_s * np;   // np
  int* order = reinterpret_cast<int*>(nrm + np);   // np
  __shared__ int s_rot;
  // blocks nsplit.. work on the second batch (A2 -> U2), same shapes
  const bool second = (int)blockIdx.x >= nsplit;
  const long long bi = second ? blockIdx.x - nsplit : blockIdx.x;
  A = (second ? A2 : A) + bi * sA;
  for (long long e = threadIdx.x; e < (long long)m * np; e += blockDim.x) {
    int c = (int)(e / m), i = (int)(e % m);
    // A row-major; with `lower`, only its lower triangle (c <= i) is read
    a[(long long)c * lda_s + i] =
        (c < n && (!lower || c <= i)) ? A[(long long)i * lda + c] : 0.0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const double tol = 2.220446049250313e-16 * (double)m;
  const int npairs = np / 2;
  const int part = threadIdx.x & (JAC_LANES - 1);
  // every lane of a warp runs the pair loop the same number of times, so the
  // shuffles below always see the whole warp
  const int slots = (npairs * JAC_LANES + blockDim.x - 1) / blockDim.x * blockDim.x;
  int sweep = 0;
  for (; sweep < JAC_MAX_SWEEPS; ++sweep) {
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    for (int rnd = 0; rnd < np - 1; ++rnd) {
      for (int t = threadIdx.x; t < slots; t += blockDim.x) {
        const int pi = t / JAC_LANES;
        const bool on = pi < npairs;
        // circle method: slot 0 fixed, others rotate
        const int s1 = pi, s2 = np - 1 - pi;
        const int p = (s1 == 0) ? 0 : 1 + (s1 - 1 + rnd) % (np - 1);
        const int q = 1 + (s2 - 1 + rnd) % (np - 1);
        double* ap = a + (long long)(on ? p : 0) * lda_s;
        double* aq = a + (long long)(on ? q : 0) * lda_s;
        double a0 = 0.0, b0 = 0.0, g0 = 0.0, a1 = 0.0, b1 = 0.0, g1 = 0.0;
        if (on) {
          int i = part;
          for (; i + JAC_LANES < m; i += 2 * JAC_LANES) {
            const double x0 = ap[i], y0 = aq[i];
            const double x1 = ap[i + JAC_LANES], y1 = aq[i + JAC_LANES];
            a0 = fma(x0, x0, a0);
            b0 = fma(y0, y0, b0);
            g0 = fma(x0, y0, g0);
            a1 = fma(x1, x1, a1);
            b1 = fma(y1, y1, b1);
            g1 = fma(x1, y1, g1);
          }
          if (i < m) {
            const double x0 = ap[i], y0 = aq[i];
            a0 = fma(x0, x0, a0);
            b0 = fma(y0, y0, b0);
            g0 = fma(x0, y0, g0);
          }
        }
        double al = a0 + a1, be = b0 + b1, ga = g0 + g1;
#pragma unroll
        for (int o = 1; o < JAC_LANES; o <<= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          ga += __shfl_xor_sync(0xffffffffu, ga, o);
        }
        if (on && ga != 0.0 && fabs(ga) > tol * sqrt(al * be)) {
          const double zeta = (be - al) / (2.0 * ga);
          double c, s;
          float tf;
          if (fabs(zeta) > 1e7) {
            // small angle: t = 1 / (2 zeta) to relative 1e-14, c^2 + s^2 = 1 + O(t^4)
            const double t = 0.5 / zeta;
            c = fma(-0.5 * t, t, 1.0);
            s = t * c;
            tf = (float)t;
          } else {
            const float zf = (float)zeta;
            tf = copysignf(1.0f, zf) / (fabsf(zf) + sqrtf(fmaf(zf, zf, 1.0f)));
            const float cf = rsqrtf(fmaf(tf, tf, 1.0f));
            c = (double)cf;
            s = (double)cf * (double)tf;
            // renormalise: (c, s) /= sqrt(1 + d), d = c^2 + s^2 - 1 ~ 1e-7
            const double d = fma(c, c, fma(s, s, -1.0));
            const double f = fma(d, fma(0.375, d, -0.5), 1.0);
            c *= f;
            s *= f;
          }
          if (s != 0.0) {
            for (int i = part; i < m; i += JAC_LANES) {
              const double x = ap[i], y = aq[i];
              ap[i] = c * x - s * y;
              aq[i] = s * x + c * y;
            }
            s_rot = 1;
          }
        }
      }
      __syncthreads();
    }
    if (!s_rot) break;
    __syncthreads();
  }
  if (threadIdx.x == 0 && sweep >= JAC_MAX_SWEEPS && info) atomicCAS(info, 0, 1);
  // column norms
  for (int c = warp; c < np; c += nwarps) {
    double s = 0.0;
    for (int i = lane; i < m; i += 32) s += a[(long long)c * lda_s + i] * a[(long long)c * lda_s + i];
    s = warp_sum(s);
    if (lane == 0) nrm[c] = sqrt(s);
  }
  __syncthreads();
  // rank of each column by decreasing norm (ties by index).  A NaN norm
  // (non-finite input) ranks below every number, so the ranks stay a
  // permutation and every order[] slot is written
  for (int c = threadIdx.x; c < np; c += blockDim.x) {
    int rk = 0;
    const double v = nrm[c] == nrm[c] ? nrm[c] : -1.0;
    for (int o = 0; o < np; ++o) {
      const double w = nrm[o] == nrm[o] ? nrm[o] : -1.0;
      rk += (w > v) || (w == v && o < c);
    }
    order[rk] = c;
  }
  __syncthreads();
  double* Ub = (second ? U2 : U) + bi * sU;
  double* svb = (sv && !second) ? sv + bi * sS : nullptr;
  const double smax = nrm[order[0]];
  const double tiny = (smax > 0.0) ? smax * 1e-150 : 1e-300;
  // normalised leading columns; columns that carry no direction are
  // completed below by Gram-Schmidt on the unit vectors
  for (int j = warp; j < r; j += nwarps) {
    const int c = min(max(order[j < np ? j : np - 1], 0), np - 1);
    double s = nrm[c];
    if (svb && lane == 0) svb[j] = (j < n) ? s : 0.0;
    bool ok = (j < n) && s > tiny;
    for (int i = lane; i < m; i += 32)
      Ub[(long long)i * ldu + j] = ok ? a[(long long)c * lda_s + i] / s : 0.0;
  }
  __syncthreads();
  // completion (rare: zero or rank-deficient input); serial over columns
  if (warp == 0) {
    for (int j = 0; j < r; ++j) {
      const int c = min(max(order[j < np ? j : np - 1], 0), np - 1);
      bool ok = (j < n) && nrm[c] > tiny;
      if (ok) continue;
      for (int e = 0; e < m; ++e) {
        // candidate e_e, orthogonalise against columns 0..j-1 (twice)
        for (int i = lane; i < m; i += 32) Ub[(long long)i * ldu + j] = (i == e) ? 1.0 : 0.0;
        __syncwarp();
        for (int pass = 0; pass < 2; ++pass)
          for (int q = 0; q < j; ++q) {
            double d = 0.0;
            for (int i = lane; i < m; i += 32) d += Ub[(long long)i * ldu + q] * Ub[(long long)i * ldu + j];
            d = warp_sum(d);
            for (int i = lane; i < m; i += 32) Ub[(long long)i * ldu + j] -= d * Ub[(long long)i * ldu + q];
            __syncwarp();
          }
        double s = 0.0;
        for (int i = lane; i < m; i += 32) s += Ub[(long long)i * ldu + j] * Ub[(long long)i * ldu + j];
        s = sqrt(warp_sum(s));
        if (s > 0.5) {
          for (int i = lane; i < m; i += 32) Ub[(long long)i * ldu + j] /= s;
          __syncwarp();
          break;
        }
      }
    }
  }
}
// Compact WY form of a factored panel of jb reflectors (LAPACK larft,
// forward, columnwise): Vc (jb x mp, row-major) holds the reflectors with
// their unit diagonal and zeros above it written out, and T (jb x jb, upper)
// satisfies H_0 H_1 ... H_{jb-1} = I - V T V^T (V = Vc^T).  One CTA per
// matrix; the panel is read from the column-major work array (column a at
// P + a * ldw, rows 0..mp-1 relative to the panel's diagonal).
constexpr int kWY = 32;   // panel width of the blocked QR
__global__ void __launch_bounds__(256)
wy_kernel(int mp, int jb, const double* __restrict__ P, int ldw, long long sW,
          const double* __restrict__ tau, long long sTau, double* __restrict__ Vc, long long sV,
          double* __restrict__ T, long long sT) {
  __shared__ double G[kWY][kWY + 1];
  __shared__ double Ts[kWY][kWY + 1];
  const long long b = blockIdx.x;
  P += b * sW;
  tau += b * sTau;
  Vc += b * sV;
  T += b * sT;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (long long e = threadIdx.x; e < (long long)jb * mp; e += blockDim.x) {
    const int a = (int)(e / mp), r = (int)(e - (long long)a * mp);
    Vc[e] = r < a ? 0.0 : (r == a ? 1.0 : P[(long long)a * ldw + r]);
  }
  // G(a, c) = v_a . v_c for a < c: v_c starts at row c (unit), v_a there
  // holds P(a, c) (a < c), both below
  for (int q = warp; q < jb * jb; q += nwarps) {
    const int a = q / jb, c = q - a * jb;
    if (a >= c) continue;
    double d = 0.0;
    for (int r = c + 1 + lane; r < mp; r += 32)
      d += P[(long long)a * ldw + r] * P[(long long)c * ldw + r];
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) G[a][c] = d + P[(long long)a * ldw + c];
  }
  __syncthreads();
  // T(i, i) = tau_i; T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i), one column
  // at a time by the first warp (lane r owns row r)
  if (warp == 0) {
    for (int i = 0; i < jb; ++i) {
      const double ti = tau[i];
      double v = 0.0;
      if (lane < i) {
        for (int c = lane; c < i; ++c) v += Ts[lane][c] * G[c][i];
        v *= -ti;
      }
      __syncwarp();
      if (lane < i) Ts[lane][i] = v;
      if (lane == i) Ts[i][i] = ti;
      if (lane > i && lane < jb) Ts[lane][i] = 0.0;
      __syncwarp();
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) T[e] = Ts[e / jb][e % jb];
}

}  // namespace

size_t qr_blocked_ws_elems(int m, int ncol, int batch) {
  return (size_t)batch * ((size_t)kWY * m + (size_t)kWY * kWY + 2 * (size_t)ncol * kWY) + 64;
}

void qr_blocked(cudaStream_t st, int m, int nfac, int ncol, double* W, int ldw, long long sW,
                double* tau, long long sTau, int batch, double* ws) {
  if (batch <= 0 || m <= 0 || nfac <= 0) return;
  if (nfac <= 2 * kWY) {
    panel_qr(st, m, nfac, ncol, W, ldw, sW, tau, sTau, batch);
    return;
  }
  SLU_REQUIRE(ws, "qr_blocked: workspace missing");
  const long long sV = (long long)kWY * m, sT = (long long)kWY * kWY, sX = (long long)ncol * kWY;
  double* Vc = ws;
  double* T = Vc + batch * sV;
  double* X1 = T + batch * sT;
  double* X2 = X1 + batch * sX;
  const int nf = std::min(nfac, m);
  for (int j0 = 0; j0 < nf; j0 += kWY) {
    const int jb = std::min(kWY, nf - j0), mp = m - j0;
    double* Pj = W + (long long)j0 * ldw + j0;
    panel_qr(st, mp, jb, jb, Pj, ldw, sW, tau + j0, sTau, batch);
    const int nc = ncol - j0 - jb;
    if (nc <= 0) continue;
    wy_kernel<<<batch, 256, 0, st>>>(mp, jb, Pj, ldw, sW, tau + j0, sTau, Vc, sV, T, sT);
    check_launch("wy_kernel");
    // trailing columns C (mp x nc, column-major: C^T row-major with ld ldw)
    // <- Q^T C, i.e. C^T <- C^T - (C^T V) T V^T
    double* Ct = Pj + (long long)jb * ldw;
    gemm_batched<double>(st, false, true, nc, jb, mp, 1.0, Ct, ldw, sW, 0, Vc, mp, sV, 0, 0.0, X1,
                         jb, sX, 0, batch);
    gemm_batched<double>(st, false, false, nc, jb, jb, 1.0, X1, jb, sX, 0, T, jb, sT, 0, 0.0, X2,
                         jb, sX, 0, batch);
    gemm_batched<double>(st, false, false, nc, mp, jb, -1.0, X2, jb, sX, 0, Vc, mp, sV, 0, 1.0, Ct,
                         ldw, sW, 0, batch);
  }
}

void panel_qr(cudaStream_t st, int m, int nfac, int ncol, double* W, int ldw, long long sW,
              double* tau, long long sTau, int batch) {
  if (batch <= 0 || m <= 0 || nfac <= 0) return;
  size_t sm = (size_t)m * ncol * sizeof(double);
  int use_smem = sm <= 200 * 1024;
  if (!use_smem) sm = 0;
  ensure_smem(reinterpret_cast<const void*>(panel_qr_kernel), sm);
  panel_qr_kernel<<<batch, 512, sm, st>>>(m, nfac, ncol, W, ldw, sW, tau, sTau, use_smem, W,
                                          tau, batch);
  check_launch("panel_qr_kernel");
}

void panel_qr2(cudaStream_t st, int m, int nfac, int ncol, double* W, double* W2, int ldw,
               long long sW, double* tau, double* tau2, long long sTau, int batch) {
  if (batch <= 0 || m <= 0 || nfac <= 0) return;
  size_t sm = (size_t)m * ncol * sizeof(double);
  int use_smem = sm <= 200 * 1024;
  if (!use_smem) sm = 0;
  ensure_smem(reinterpret_cast<const void*>(panel_qr_kernel), sm);
  panel_qr_kernel<<<2 * batch, 512, sm, st>>>(m, nfac, ncol, W, ldw, sW, tau, sTau, use_smem,
                                              W2, tau2, batch);
  check_launch("panel_qr_kernel");
}

void apply_q(cudaStream_t st, bool transpose, int m, int k, const double* V, int ldv,
             long long sV, const double* tau, long long sTau, double* C, int ldc, long long sC,
             int nc, int batch) {
  if (batch <= 0 || nc <= 0 || m <= 0) return;
  dim3 grid((nc + 7) / 8, batch);
  apply_q_kernel<<<grid, 256, 0, st>>>(transpose, m, k, V, ldv, sV, tau, sTau, C, ldc, sC, nc);
  check_launch("apply_q_kernel");
}

void jacobi_left_sv(cudaStream_t st, int m, int n, const double* A, int lda, long long sA, int r,
                    double* U, int ldu, long long sU, double* sv, long long sS, int batch,
                    int* info, bool lower) {
  if (batch <= 0 || r <= 0) return;
  SLU_REQUIRE(r <= m, "jacobi: rank larger than rows");
  int np = n + (n & 1);
  size_t sm = (size_t)(m | 1) * np * sizeof(double) + np * sizeof(double) + np * sizeof(int);
  SLU_REQUIRE(sm <= 220 * 1024, "jacobi: block too large for shared memory");
  ensure_smem(reinterpret_cast<const void*>(jacobi_kernel), sm);
  int threads = 32 * std::min(32, std::max(2, (np / 2 * JAC_LANES + 31) / 32));
  jacobi_kernel<<<batch, threads, sm, st>>>(m, n, A, lda, sA, r, U, ldu, sU, sv, sS, info,
                                            lower ? 1 : 0, A, U, batch);
  check_launch("jacobi_kernel");
}

void jacobi_left_sv2(cudaStream_t st, int m, int n, const double* A, const double* A2, int lda,
                     long long sA, int r, double* U, double* U2, int ldu, long long sU, int batch,
                     int* info, bool lower) {
  if (batch <= 0 || r <= 0) return;
  SLU_REQUIRE(r <= m, "jacobi: rank larger than rows");
  int np = n + (n & 1);
  size_t sm = (size_t)(m | 1) * np * sizeof(double) + np * sizeof(double) + np * sizeof(int);
  SLU_REQUIRE(sm <= 220 * 1024, "jacobi: block too large for shared memory");
  ensure_smem(reinterpret_cast<const void*>(jacobi_kernel), sm);
  int threads = 32 * std::min(32, std::max(2, (np / 2 * JAC_LANES + 31) / 32));
  jacobi_kernel<<<2 * batch, threads, sm, st>>>(m, n, A, lda, sA, r, U, ldu, sU, nullptr, 0, info,
                                                lower ? 1 : 0, A2, U2, batch);
  check_launch("jacobi_kernel");
}

}  // namespace slu
