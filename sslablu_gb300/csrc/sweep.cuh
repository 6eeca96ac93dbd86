// One tree step of the ULV solve as a block-sparse product (mode N).
//
// The forward, root and backward steps of ULVsparse.solve (matAssembly/HBS/
// ULVsparse.py:296-327) are each linear in the vectors a block reads, so the
// factors of one block compose, at factor time, into one dense operator S_b
// (hbs_make_sweep, sweep_ops.cu):
//   forward  [ru; x_parent] = Q_b^T x_b                      S_b = Q_b^T
//   root     [y; v]         = [R^{-1} Q^T; D R^{-1} Q^T] x
//   backward [y_new; v_new] = [G_b; H_b] [ru; v; y_next]
//            G_b = W1 R11^{-1} [I | -Uu | -R12] + [0 | 0 | W2]
//            H_b = D_b G_b + [0 | U_b | 0]
// (W = [W1 W2] by columns nu | k, R = [R11 R12]).  The leaf level keeps
// only G (its y_new is the solution).  Every output row of every block is
// then an independent dot product of length w, so a step splits over blocks,
// row slices and column chunks -- enough CTAs to fill the GPU even for a
// handful of right-hand sides -- and a CTA runs one batch of asynchronous
// copies, one barrier, and one product: no triangular solve and no chain of
// dependent matrix-vector products inside a level.
//
// A step reads the z vector of a block from up to three row ranges of device
// arrays (the first optionally through a row permutation, the tree ordering
// of the caller's right-hand sides) and writes output rows [0, split) to one
// array (optionally through a permutation) and the rest to another.
#pragma once

#include <cstdint>

#include "dfloat.cuh"

namespace slu {
namespace sweep {

template <typename T>
struct Step {
  const T* S;          // S_b = S + b * sS: rows x w, row-major, leading dimension w
  long long sS;
  int rows, w;
  int nb, rch, nrch;   // blocks; rows per CTA slice; slices per block
  int c, cpb;          // right-hand-side columns; columns per CTA
  int nin;             // input ranges of z (1..3), concatenated in order
  const T* in_p[3];
  long long in_ld[3], in_blk[3];   // leading dimension; rows per block
  int in_rows[3];
  const int64_t* in_perm;          // input 0: row b*in_blk[0] + i read at perm[...]
  int split;                       // output rows [0, split) -> out 0, rest -> out 1
  T* out_p[2];
  long long out_ld[2], out_blk[2];
  const int64_t* out_perm;         // output 0: row b*out_blk[0] + i written at perm[...]
};

// Lanes per dot product: each sums every ks-th term of its row, then a
// butterfly of shuffles adds the ks partial sums.  Depends only on the
// element type and the dot product length, so the summation order of an
// output does not depend on the right-hand-side count or on the chunking.
// float64: two lanes (the butterfly's adds run on the FP64 pipe, which
// bounds the large levels); float32 and double-float: four.
template <typename T>
__host__ __device__ inline int split_for(int w) {
  return w >= 32 ? 4 : (w >= 8 ? 2 : 1);
}
template <>
__host__ __device__ inline int split_for<double>(int w) {
  return w >= 16 ? 2 : 1;
}

// Pitch of the transposed z tile (zT[cc][j]): congruent to ks modulo the
// elements of a 128-byte shared-memory row, so the ks lanes of one output
// and the 128/(ks*sizeof(T)) outputs of a wavefront touch distinct banks.
__host__ __device__ inline int z_pitch(int w, int ks, int elem) {
  const int q = 128 / elem;
  int p = w;
  while (p % q != ks % q) ++p;
  return p;
}

template <typename T>
__host__ __device__ inline size_t step_smem_elems(int rch, int w, int cpb, int ks) {
  return (size_t)rch * w + (size_t)cpb * z_pitch(w, ks, (int)sizeof(T));
}

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Programmatic dependent launch (sm_90 and later): wait until the grids this
// launch depends on have completed and their writes are visible (returns at
// once for a launch without such a dependency); allow the next launch of the
// stream to begin scheduling its CTAs.
__device__ __forceinline__ void grid_dependency_wait() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
}
__device__ __forceinline__ void launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  if (sizeof(T) == 8) cp_async8(dst, src);
  else cp_async4(dst, src);
}

// Contiguous global -> shared copy of `bytes` bytes (a multiple of the
// element size): 16-byte copies when both ends are 16-byte aligned.
template <typename T>
__device__ __forceinline__ void copy_contig(T* dst, const T* src, size_t count) {
  const size_t bytes = count * sizeof(T);
  if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
    const size_t n16 = bytes >> 4;
    const char* s = reinterpret_cast<const char*>(src);
    char* d = reinterpret_cast<char*>(dst);
    for (size_t e = threadIdx.x; e < n16; e += blockDim.x) cp_async16(d + 16 * e, s + 16 * e);
    const size_t done = n16 * 16 / sizeof(T);
    for (size_t e = done + threadIdx.x; e < count; e += blockDim.x) cp_async_elem(dst + e, src + e);
  } else {
    for (size_t e = threadIdx.x; e < count; e += blockDim.x) cp_async_elem(dst + e, src + e);
  }
}

// Products of R interleaved items per thread (independent accumulation
// chains): item t -> output (i, cc), lane part t % KS.  The full-width case
// (all R items of the warp present) runs without per-item guards.
template <typename T, int R, int KS>
__device__ __forceinline__ void product(const Step<T>& s, const T* Ss, const T* zT, int pz, int b,
                                        int r0, int nr, int c0, int nc) {
  constexpr int LKS = KS == 8 ? 3 : (KS == 4 ? 2 : (KS == 2 ? 1 : 0));
  const int w = s.w, items = nr * nc * KS, lane = threadIdx.x & 31;
  const int part = lane & (KS - 1);
  const int nterm = (w - part + KS - 1) / KS;
  const int stride = blockDim.x;
  for (int base = threadIdx.x - lane; base < items; base += R * stride) {
    const T* sp[R];
    const T* zp[R];
    int i[R], cc[R];
    bool on[R];
    int nact = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int t = base + r * stride + lane;
      on[r] = t < items;
      const int e = t >> LKS;
      const int ii = on[r] ? e / nc : 0;
      i[r] = ii;
      cc[r] = on[r] ? e - ii * nc : 0;
      sp[r] = Ss + ii * w + part;
      zp[r] = zT + cc[r] * pz + part;
      if (base + r * stride < items) nact = r + 1;   // warp-uniform
    }
    DotAcc<T> da[R];
#pragma unroll
    for (int r = 0; r < R; ++r) da[r].zero();
    if (nact == R) {
#pragma unroll 4
      for (int m = 0; m < nterm; ++m) {
#pragma unroll
        for (int r = 0; r < R; ++r) da[r].add(sp[r][m * KS], zp[r][m * KS]);
      }
    } else {
      for (int m = 0; m < nterm; ++m) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r < nact) da[r].add(sp[r][m * KS], zp[r][m * KS]);
      }
    }
    T acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = da[r].value();
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r < nact) {
#pragma unroll
        for (int o = KS >> 1; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
        if (on[r] && part == 0) {
          const int row = r0 + i[r];
          const int col = c0 + cc[r];
          if (row < s.split) {
            const long long q = (long long)b * s.out_blk[0] + row;
            const long long dst = s.out_perm ? __ldg(s.out_perm + q) : q;
            s.out_p[0][dst * s.out_ld[0] + col] = acc[r];
          } else {
            const long long q = (long long)b * s.out_blk[1] + (row - s.split);
            s.out_p[1][q * s.out_ld[1] + col] = acc[r];
          }
        }
      }
    }
  }
}

template <typename T, int KS>
__device__ __forceinline__ void product_ks(const Step<T>& s, const T* Ss, const T* zT, int pz,
                                           int b, int r0, int nr, int c0, int nc) {
  const int per = (nr * nc * KS + blockDim.x - 1) / blockDim.x;
  if (per >= 4) product<T, 4, KS>(s, Ss, zT, pz, b, r0, nr, c0, nc);
  else if (per >= 2) product<T, 2, KS>(s, Ss, zT, pz, b, r0, nr, c0, nc);
  else product<T, 1, KS>(s, Ss, zT, pz, b, r0, nr, c0, nc);
}

// CTA (xb, cy) of a step: block b = xb / nrch, row slice xb % nrch, column
// chunk cy.
template <typename T>
__device__ __forceinline__ void step_body(const Step<T>& s, unsigned char* sm_raw, int xb, int cy) {
  const int b = xb / s.nrch;
  const int r0 = (xb - b * s.nrch) * s.rch;
  const int nr = min(s.rch, s.rows - r0);
  const int c0 = cy * s.cpb, nc = min(s.cpb, s.c - c0);
  if (nr <= 0 || nc <= 0) return;   // uniform over the CTA
  const int w = s.w, ks = split_for<T>(w), pz = z_pitch(w, ks, (int)sizeof(T));
  T* Ss = reinterpret_cast<T*>(sm_raw);      // nr x w (rows r0.. of S_b)
  T* zT = Ss + (size_t)s.rch * w;            // nc x pz, zT[cc][j] = z[j][c0 + cc]
  // the block operator is constant: its copy starts before the wait for the
  // previous launch of the stream (programmatic dependent launch), whose
  // outputs are the z vectors read next
  copy_contig(Ss, s.S + (size_t)b * s.sS + (size_t)r0 * w, (size_t)nr * w);
  grid_dependency_wait();
  // z: element (j, cc) with cc fastest (coalesced global reads)
  int j0 = 0;
  for (int q = 0; q < s.nin; ++q) {
    const int rows = s.in_rows[q];
    const T* p = s.in_p[q];
    const long long ld = s.in_ld[q], rb = (long long)b * s.in_blk[q];
    const int64_t* perm = q == 0 ? s.in_perm : nullptr;
    const int total = rows * nc;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      const int jj = e / nc, cc = e - jj * nc;
      const long long row = perm ? __ldg(perm + rb + jj) : rb + jj;
      cp_async_elem(zT + cc * pz + j0 + jj, p + row * ld + c0 + cc);
    }
    j0 += rows;
  }
  cp_async_wait();
  __syncthreads();
  // inputs staged: the next launch may start its own operator copies
  launch_dependents();
  if (ks == 4) product_ks<T, 4>(s, Ss, zT, pz, b, r0, nr, c0, nc);
  else if (ks == 2) product_ks<T, 2>(s, Ss, zT, pz, b, r0, nr, c0, nc);
  else product_ks<T, 1>(s, Ss, zT, pz, b, r0, nr, c0, nc);
}

}  // namespace sweep
}  // namespace slu
