// Slab source-target maps of the stencil discretisation, applied on the GPU
// by solves of the slab interiors.
//
// Upstream forms the interface couplings of the overlapping multislab method
// as linear operators (multislab/oms.py:96-125, oms.compute_stmaps):
//
//   S_J g = (A_ii^{-1} A_ib[:, J] g)[Ic],   S_J^T y = A_ib[:, J]^T A_ii^{-T} (y on Ic)
//
// with A_ii the interior rows of the stencil operator on a double-wide slab
// (solver/stencil/stencilSolver.py:40-120 in 2-D, 221-420 in 3-D; upstream
// factors it with scipy's sparse LU, stencilSolver.solver_Aii), A_ib its
// couplings to the slab's edge planes J (left Il / right Ir) and Ic the
// interior points on the slab's centre plane.  The randomized HBS assembly
// samples them (matAssembly/matAssembler.py:112-117: Y = S Om, Z = S^T Psi).
//
// Here every slab of a batch and every column of a block of right-hand sides
// is solved at once by the Chebyshev semi-iterative method (Golub and Varga,
// "Chebyshev semi-iterative methods ...", Numer. Math. 3, 1961) on
// M = -A_ii, which is symmetric positive definite when the slab is thin
// enough for the Helmholtz shift: with c11 = c22 = c33 = 1 and zeroth-order
// term kappa^2 c(x), the spectrum of M lies in
//   [sum_a 4/h_a^2 sin^2(pi / (2 (n_a + 1))) - kappa^2 c_max,
//    sum_a 4/h_a^2 sin^2(pi n_a / (2 (n_a + 1))) - kappa^2 c_min]
// (the separable Dirichlet Laplacian's extreme eigenvalues, shifted by the
// diagonal's range: Weyl's inequalities).  With those bounds the error after
// k steps is at most 2 rho^k of the solution (rho = (sqrt(kappa_M) - 1) /
// (sqrt(kappa_M) + 1)), so the step count for a requested relative accuracy
// is fixed in advance; no inner products are needed, and each step is one
// stencil application fused with the three-term update:
//   x_{k+1} = w_{k+1} (x_k - x_{k-1} + gamma (b - M x_k)) + x_{k-1}.
// Slabs whose lower bound is not positive (a Helmholtz shift above the
// slab's smallest Laplacian eigenvalue) are refused.
//
// Layout: unknowns of slab s at interior point p = (iy * nzi + iz) * nxi + ix
// (x fastest; nzi = 1 in 2-D), column c: element ((s * NP + p) * C + c), so
// a warp reads 32 consecutive columns of one point.
#include <cmath>

#include "abi_types.cuh"
#include "hbs.cuh"

namespace slu {
namespace slab {

struct Geom {
  int nxi, nyi, nzi;    // interior points along x, y, z (nzi = 1 in 2-D)
  double ihx2, ihy2, ihz2;   // 1 / h^2 (ihz2 = 0 in 2-D)
  double hx, hy, hz;
  double kappa2;        // kappa^2 of the zeroth-order term kappa^2 c(x)
  int coef;             // 0: c = 1; 1: c = 1 + 0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z)
  long long NP;         // interior points per slab
};

// diag[s][p] = M_pp = 2/hx^2 + 2/hy^2 (+ 2/hz^2) - kappa^2 c(x_p)
__global__ void diag_kernel(const Geom g, int nslabs, const double* __restrict__ x0,
                            double* __restrict__ diag) {
  const long long total = (long long)nslabs * g.NP;
  const double base = 2.0 * (g.ihx2 + g.ihy2 + g.ihz2);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long s = e / g.NP, p = e - s * g.NP;
    double c = 1.0;
    if (g.coef == 1) {
      const int ix = (int)(p % g.nxi);
      const long long q = p / g.nxi;
      const int iz = (int)(q % g.nzi), iy = (int)(q / g.nzi);
      const double x = x0[s] + g.hx * (ix + 1), y = g.hy * (iy + 1), z = g.hz * (iz + 1);
      c = 1.0 + 0.5 * sin(2.0 * M_PI * x) * sin(2.0 * M_PI * y) * sin(2.0 * M_PI * z);
    }
    diag[e] = base - g.kappa2 * c;
  }
}

// One Chebyshev step for every slab and column.  b: forward (trans = 0)
// -XL / hx^2 on plane ix = 0 and -XR / hx^2 on plane ix = nxi - 1 (the edge
// data through A_ib); transposed -X on the centre plane.  xn holds x_{k-1}
// on entry and x_{k+1} on exit; the first step (x_0 = 0) writes gamma b.
__global__ void cheb_step_kernel(const Geom g, int nslabs, int C, const double* __restrict__ diag,
                                 const double* __restrict__ xc, double* __restrict__ xn,
                                 double om, double gam, int first, const double* __restrict__ XL,
                                 const double* __restrict__ XR, long long ldx, int trans) {
  const long long NP = g.NP;
  const long long total = (long long)nslabs * NP * C;
  const long long m = NP / g.nxi;          // points per plane
  const int ic = (g.nxi - 1) / 2;
  const long long sz = (long long)g.nxi * C, sy = (long long)g.nxi * g.nzi * C;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long t = e / C;
    const int col = (int)(e - t * C);
    const long long s = t / NP, p = t - s * NP;
    const int ix = (int)(p % g.nxi);
    const long long q = p / g.nxi;          // plane index iy * nzi + iz
    const int iz = (int)(q % g.nzi), iy = (int)(q / g.nzi);
    double b = 0.0;
    const long long src = (s * m + q) * ldx + col;
    if (!trans) {
      if (ix == 0 && XL) b -= XL[src] * g.ihx2;
      if (ix == g.nxi - 1 && XR) b -= XR[src] * g.ihx2;
    } else if (ix == ic) {
      b = -XL[src];
    }
    if (first) {
      xn[e] = gam * b;
      continue;
    }
    const double xv = xc[e];
    double nb = 0.0;
    if (ix > 0) nb += g.ihx2 * xc[e - C];
    if (ix < g.nxi - 1) nb += g.ihx2 * xc[e + C];
    if (iz > 0) nb += g.ihz2 * xc[e - sz];
    if (iz < g.nzi - 1) nb += g.ihz2 * xc[e + sz];
    if (iy > 0) nb += g.ihy2 * xc[e - sy];
    if (iy < g.nyi - 1) nb += g.ihy2 * xc[e + sy];
    const double Mx = fma(diag[s * NP + p], xv, -nb);
    const double xp = xn[e];
    xn[e] = fma(om, xv - xp + gam * (b - Mx), xp);
  }
}

// Y_s[q, c] = x[s, (q, ix = plane), c] * scale for every slab.
__global__ void take_plane_kernel(const Geom g, int nslabs, int C, const double* __restrict__ x,
                                  int plane, double scale, double* __restrict__ Y, long long ldy) {
  const long long m = g.NP / g.nxi;
  const long long total = (long long)nslabs * m * C;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long t = e / C;
    const int col = (int)(e - t * C);
    const long long s = t / m, q = t - s * m;
    Y[(s * m + q) * ldy + col] = scale * x[((s * g.NP) + q * g.nxi + plane) * C + col];
  }
}

double lap_eig(int n, double ih2, bool top) {
  const double a = M_PI * (top ? n : 1) / (2.0 * (n + 1));
  const double sn = std::sin(a);
  return 4.0 * ih2 * sn * sn;
}

unsigned grid_for(long long n) {
  const long long b = (n + 255) / 256;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, (long long)num_sms() * 16));
}

}  // namespace slab
}  // namespace slu

extern "C" int slu_slab_maps_apply(slu_handle_t h, int nx, int ny, int nz, double width,
                                   double kappa, int coef, int nslabs, const double* x0,
                                   const double* XL, const double* XR, int ldx, double* YL,
                                   double* YR, int ldy, int ncols, int trans, double tol,
                                   int* steps_out) {
  return slu::guard_call(h, [&] {
    using namespace slu;
    SLU_REQUIRE(h && x0, "null argument");
    SLU_REQUIRE(nx >= 3 && nx % 2 == 1, "nx must be odd and >= 3 (the centre plane is a grid plane)");
    SLU_REQUIRE(ny >= 3 && (nz == 0 || nz >= 3), "ny >= 3 and nz == 0 (2-D) or nz >= 3");
    SLU_REQUIRE(width > 0.0 && nslabs >= 1 && ncols >= 1 && ldx >= ncols && ldy >= ncols,
                "bad slab geometry or block shape");
    SLU_REQUIRE(coef == 0 || coef == 1, "coef must be 0 (constant) or 1 (the C3 coefficient)");
    SLU_REQUIRE(tol > 0.0 && tol < 1.0, "tol must lie in (0, 1)");
    if (!trans) {
      SLU_REQUIRE(YL && (XL || XR), "forward apply needs an output and at least one input");
    } else {
      SLU_REQUIRE(XL && (YL || YR), "transposed apply needs an input and at least one output");
    }
    slab::Geom g{};
    g.nxi = nx - 2;
    g.nyi = ny - 2;
    g.nzi = nz == 0 ? 1 : nz - 2;
    g.hx = width / (nx - 1);
    g.hy = 1.0 / (ny - 1);
    g.hz = nz == 0 ? 0.0 : 1.0 / (nz - 1);
    g.ihx2 = 1.0 / (g.hx * g.hx);
    g.ihy2 = 1.0 / (g.hy * g.hy);
    g.ihz2 = nz == 0 ? 0.0 : 1.0 / (g.hz * g.hz);
    g.kappa2 = kappa * kappa;
    g.coef = coef;
    g.NP = (long long)g.nxi * g.nyi * g.nzi;
    double lmin = slab::lap_eig(g.nxi, g.ihx2, false) + slab::lap_eig(g.nyi, g.ihy2, false);
    double lmax = slab::lap_eig(g.nxi, g.ihx2, true) + slab::lap_eig(g.nyi, g.ihy2, true);
    if (nz != 0) {
      lmin += slab::lap_eig(g.nzi, g.ihz2, false);
      lmax += slab::lap_eig(g.nzi, g.ihz2, true);
    }
    const double cmin = coef == 1 ? 0.5 : 1.0, cmax = coef == 1 ? 1.5 : 1.0;
    lmin -= g.kappa2 * cmax;
    lmax -= g.kappa2 * cmin;
    SLU_REQUIRE(lmin > 0.0,
                "slab interior operator is not definite (the Helmholtz shift exceeds the "
                "slab's smallest Laplacian eigenvalue): use thinner slabs or a smaller kappa");
    const double kap = lmax / lmin;
    const double rho = (std::sqrt(kap) - 1.0) / (std::sqrt(kap) + 1.0);
    const int steps = rho <= 0.0 ? 1 : (int)std::ceil(std::log(2.0 / tol) / -std::log(rho));
    SLU_REQUIRE(steps <= 100000, "slab solve would need more than 1e5 Chebyshev steps");
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double sig = delta / theta, gam = 1.0 / theta;
    cudaStream_t st = h->h.stream;
    const long long nel = (long long)nslabs * g.NP * ncols;
    const size_t vbytes = ((size_t)nel * 8 + 255) & ~size_t(255);
    const size_t dbytes = (((size_t)nslabs * g.NP * 8) + 255) & ~size_t(255);
    h->h.ws.reserve(2 * vbytes + dbytes + 256, st);
    double* xa = h->h.ws.take<double>(nel);
    double* xb = h->h.ws.take<double>(nel);
    double* diag = h->h.ws.take<double>((size_t)nslabs * g.NP);
    DevBuf x0d;
    x0d.alloc(8 * (size_t)nslabs, st);
    SLU_CHECK_CUDA(cudaMemcpyAsync(x0d.p, x0, 8 * (size_t)nslabs, cudaMemcpyHostToDevice, st));
    slab::diag_kernel<<<slab::grid_for((long long)nslabs * g.NP), 256, 0, st>>>(
        g, nslabs, x0d.as<double>(), diag);
    check_launch("slab diag_kernel");
    // x_1 = gamma b into xb; then x_{k+1} overwrites x_{k-1}
    const double* inL = XL;
    const double* inR = trans ? nullptr : XR;
    slab::cheb_step_kernel<<<slab::grid_for(nel), 256, 0, st>>>(
        g, nslabs, ncols, diag, nullptr, xb, 1.0, gam, 1, inL, inR, ldx, trans);
    check_launch("slab cheb_step_kernel");
    SLU_CHECK_CUDA(cudaMemsetAsync(xa, 0, 8 * (size_t)nel, st));
    double* cur = xb;   // x_k
    double* prev = xa;  // x_{k-1}
    double om = 1.0;
    for (int k = 1; k < steps; ++k) {
      om = (k == 1) ? 1.0 / (1.0 - 0.5 * sig * sig) : 1.0 / (1.0 - 0.25 * sig * sig * om);
      slab::cheb_step_kernel<<<slab::grid_for(nel), 256, 0, st>>>(
          g, nslabs, ncols, diag, cur, prev, om, gam, 0, inL, inR, ldx, trans);
      check_launch("slab cheb_step_kernel");
      std::swap(cur, prev);
    }
    const long long ntake = (long long)nslabs * (g.NP / g.nxi) * ncols;
    if (!trans) {
      slab::take_plane_kernel<<<slab::grid_for(ntake), 256, 0, st>>>(
          g, nslabs, ncols, cur, (g.nxi - 1) / 2, 1.0, YL, ldy);
      check_launch("slab take_plane_kernel");
    } else {
      if (YL) {
        slab::take_plane_kernel<<<slab::grid_for(ntake), 256, 0, st>>>(g, nslabs, ncols, cur, 0,
                                                                       g.ihx2, YL, ldy);
        check_launch("slab take_plane_kernel");
      }
      if (YR) {
        slab::take_plane_kernel<<<slab::grid_for(ntake), 256, 0, st>>>(
            g, nslabs, ncols, cur, g.nxi - 1, g.ihx2, YR, ldy);
        check_launch("slab take_plane_kernel");
      }
    }
    if (steps_out) *steps_out = steps;   // x0d is freed in stream order on return
  });
}
