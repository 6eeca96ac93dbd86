// Tensor-core ULV sweep and HBS apply: every step product on tcgen05 with
// error-free bfloat16 digit splitting.
//
// The mode-N solve (ULVsparse.solve, matAssembly/HBS/ULVsparse.py:296-327)
// and the HBS apply (HBSnew.HBSMAT.matmat, matAssembly/HBS/HBSnew.py:308-350)
// run here as the same block-sparse steps as the float64 step kernels
// (sweep.cuh, sweep_host.cuh): out_b = S_b z_b per block, z_b gathered from up
// to three row ranges.  Each product is evaluated to float64-level accuracy
// from bfloat16 tensor-core products, by the error-free splitting scheme of
// Ozaki, Ogita, Oishi and Rump ("Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication", Numer.
// Algorithms 59, 2012), in the form used on tensor cores by Mukunoki, Ozaki,
// Ogita and Imamura (ISC 2020):
//
//   * every row i of S_b is scaled by a power of two 2^E_i (max |row| <
//     2^(E_i - 1): scaled rows lie below 1/2) and written as seven balanced
//     base-256 digits, S_ik = 2^E_i sum_s a_s,ik 2^(-8 (s + 1)), |a_s| <= 128
//     (factor time, float64; 55 significant bits);
//   * every column j of z_b is scaled by 2^F_j (below 1/2 again) and split
//     the same way in the kernel, from the double-float (or float64) input,
//     with float32 error-free extraction (x + sigma - sigma, sigma = 1.5 2^p)
//     and two exact TwoSum merges of the low word: seven digits z_t,
//     |z_3| <= 256 (counting from 0), the others <= 128;
//   * for every digit pair with s + t <= 8 (28 products) the tensor cores form
//     A_s Z_t in float32; all pairs of one diagonal d = s + t go into one TMEM
//     accumulator.  Every term of accumulator d is an integer multiple of
//     2^(-8 d) and, for steps of at most 128 columns (K), every partial sum
//     stays below 2^24 such units, so float32 accumulation is exact;
//   * the epilogue adds the seven diagonals exactly, in float32 (TwoSums and
//     additions whose results provably fit their grid: the diagonals lie on
//     nested 2^-8d grids with known bounds, see diag_sum), rounds once to a
//     float32 pair (or a float64 for the caller's output) and scales by
//     2^(E_i + F_j).  The exact sum matters: a residual b - A x cancels
//     ~10^3-fold, and a rounded summation of the diagonals would keep only
//     2^-48 of the largest one.
// The dropped digit pairs and the truncated digits leave a relative error of
// about 2^-55 of |S| |z| per product: float64-level.  Vectors between steps
// are double-float pairs (8 bytes, ~48 bits), so no step uses the float64
// pipe; only a float64 input is split and a float64 output assembled.
//
// Kernel (one CTA per block, row tile of NT <= 64 operator rows and 128
// right-hand-side columns; 16 digitiser warps + 1 MMA warp, one CTA per SM):
//   1. one bulk copy (cp.async.bulk, mbarrier complete_tx) brings the seven
//      operator digit images, stored in global memory already in the
//      core-matrix order the MMA reads (8 x 8 bf16 tiles of 128 bytes,
//      K-major, no swizzle), before the wait for the previous launch;
//   2. griddepcontrol.wait (programmatic dependent launch); the digitiser
//      warps find each column's largest magnitude (four threads per column,
//      8 loads in flight each), then digitise z chunk by chunk (32 k) into
//      two chunk buffers of seven 128 x 32 digit images;
//   3. the MMA warp issues tcgen05.mma.kind::f16 (M = 128 columns, N = NT
//      rows, K = 16) for the 28 digit pairs of each chunk into seven TMEM
//      accumulators of NT columns as soon as the chunk is written, and hands
//      the buffer back with tcgen05.commit: chunk c + 1 is digitised while
//      the tensor cores work on chunk c;
//   4. the digitiser warps read the accumulators (tcgen05.ld), combine,
//      scale and store (one thread per column: coalesced rows); float64
//      outputs are assembled from the float32 pair with integer operations.
// Every mbarrier wait is bounded (2^22 polls); on a timeout the kernel sets
// the handle's device error word, waits (bounded) for its own copies, frees
// its TMEM and returns.
#include <cuda_bf16.h>

#include "hbs.cuh"
#include "sweep_host.cuh"

namespace slu {
namespace oz {

constexpr int kDig = 7;           // digits per operand
constexpr int kM = 128;           // right-hand-side columns per CTA (MMA M)
constexpr int kMaxW = 128;        // widest step whose diagonal sums stay exact in float32
constexpr int kMaxNT = 64;        // operator rows per CTA (MMA N)
constexpr int kKC = 32;           // k per digitised chunk of z (two chunk buffers)
constexpr int kDigWarps = 16;     // digitise z
constexpr int kEpiWarps = 8;      // read the accumulators, combine, store (2 per lane quadrant)
constexpr int kMmaWarp = kDigWarps + kEpiWarps;   // issues the tensor-core MMAs
constexpr int kThreads = 32 * (kMmaWarp + 1);
constexpr long long kWaitLimit = 1LL << 22;

struct OzStep {
  sweep::Step<dfloat> s;   // geometry and vectors (s.S unused)
  const uint16_t* dig;     // digit images: [Nb][ntile][kDig][NT * wP] bf16
  const float* rsc;        // row scales: [Nb][ntile * NT]
  int NT, wP, ntile;
  int in_f64;              // input range 0 holds float64 values (the caller's)
  int out_f64;             // output 0 receives float64 values (the caller's)
  // per-column normalisation of the caller's vectors: colbits[j] holds the
  // high word of the float64 bits of max_i |X_ij| over the whole column;
  // float64 inputs enter scaled by 2^-s_j (m_j < 2^s_j) and float64 outputs
  // leave scaled by 2^s_j, so every vector between steps stays near unit
  // magnitude, inside the float32 exponent range, whatever the float64 scale
  const unsigned* colbits;
  unsigned* err;           // device error word (timeouts)
  // residual form of the float64 output (the refinement's last apply step):
  // with resb set, the caller's rows receive resb - (S z) instead of S z
  // (resb in the output's layout and leading dimension), and rnorm2[j]
  // accumulates the squared 2-norm of column j of that residual (atomics;
  // zeroed by the caller)
  const double* resb;
  double* rnorm2;
};

// s_j of a column from its max-magnitude bits (0 for a zero column):
// max < 2^s_j.
__device__ __forceinline__ int col_shift(unsigned bits) {
  return bits == 0 ? 0 : min(1023, (int)((bits >> 20) & 0x7FF) - 1022);
}

// Dynamic shared memory: two z chunk buffers (seven 128 x 32 digit images
// each) and the seven NT x wP operator digit images, 1 KB alignment slack.
__host__ __device__ inline size_t smem_bytes(int NT, int wP) {
  return 2 * (size_t)kDig * kM * kKC * 2 + (size_t)kDig * NT * wP * 2 + 1024;
}

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait for the phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t addr = smem_u32(bar);
  for (long long i = 0; i < kWaitLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Contiguous global -> shared bulk copy completing on an mbarrier.
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Shared-memory matrix descriptor, K-major, no swizzle: core matrices of
// 8 rows x 16 bytes; lbo = bytes between core matrices adjacent in K,
// sbo = bytes between 8-row groups.
__device__ __forceinline__ uint64_t desc_noswz(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version
  return d;                 // base offset 0, swizzle none
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}

// ---------------------------------------------------------------- arithmetic
// x rounded to a multiple of ulp(sig) (|x| < sig / 3): Ozaki's extraction.
__device__ __forceinline__ float extract(float x, float sig) {
  return __fsub_rn(__fadd_rn(x, sig), sig);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// x 2^-sh as float32 pair (h, l), with integer operations only (no float64
// pipe): h is the scaled x with its mantissa cut to 24 bits, l the remaining
// 29 bits rounded to float32 (48 significant bits in all).  The shift is
// applied to the exponent, so it is exact; results below 2^-126 become 0
// (after normalisation these are below 2^-126 of the column's largest entry).
__device__ __forceinline__ void f64_split(double x, int sh, float& h, float& l) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sgn = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7FF) - sh;   // biased exponent of x 2^-sh
  const int fe = e - 1023 + 127;
  if (((b >> 52) & 0x7FF) == 0 || fe <= 0) {
    h = 0.f;
    l = 0.f;
    return;
  }
  if (fe >= 255) {   // beyond float32: propagate as infinity
    h = __uint_as_float(sgn | 0x7F800000u);
    l = 0.f;
    return;
  }
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  h = __uint_as_float(sgn | ((unsigned)fe << 23) | (unsigned)(mant >> 29));
  const unsigned low = (unsigned)(mant & 0x1FFFFFFFull);
  // low * 2^(e - 1075) in two exact power-of-two steps (2^-64, then
  // 2^(e - 1011)), so neither factor leaves the float32 range early
  const int pe = e - 1011 + 127;
  const float lo = pe >= 1 ? __fmul_rn(__fmul_rn(__uint2float_rn(low), 0x1p-64f),
                                       __uint_as_float((unsigned)min(pe, 254) << 23))
                           : 0.f;
  l = sgn ? -lo : lo;
}

// The seven digit diagonals a_0..a_6 summed with no rounding error, as four
// float32 terms v = h + l + e + f.  After the row and column scaling every
// operator and vector entry is below 1/2 in magnitude (|v| < K / 4 <= 2^5),
// so with K <= 128 and the digit bounds above, a_d is an integer multiple of
// 2^-(8d+16) with |a_0| < 2^5, |a_1| < 2^-2, |a_2| < 2^-9.4, |a_3| < 2^-16.7,
// |a_4| < 2^-24.4, |a_5| < 2^-32.2, |a_6| <= 2^-40 (at most 2^24 units of its
// grid each: exact float32 accumulation).  Alternating TwoSums (exact by
// construction) with plain additions whose results provably fit in 24 bits
// of their grid:
//   (h, l) = TwoSum(a_0, a_1):  l a multiple of 2^-24, |l| <= ulp(h)/2 <= 2^-19
//   l + a_2:  grid 2^-32, magnitude < 2^-9.3: exact
//   (l, e) = TwoSum(l, a_3):    e a multiple of 2^-40, |e| <= 2^-33
//   e + a_4:  grid 2^-48, magnitude < 2^-24.3: exact
//   (e, f) = TwoSum(e, a_5):    f a multiple of 2^-56, |f| <= 2^-48
//   f + a_6:  grid 2^-64, magnitude <= 2^-40 (1 + 2^-8): exact but for one
//             unit of 2^-64 at the extreme bound (~2^-69 of |v|'s bound).
// The digit products cancel heavily when |S z| is much smaller than
// |S| |z| (the apply inside a residual b - A x), so no rounding may happen
// before the sum is complete; the only rounding is the final one to a
// float32 pair or a float64 (~2^-48 of |v| for the pair).
// Then v as a float32 pair (H + Lo, |Lo| <= ulp(H) / 2): h + l may cancel,
// so H takes e in with a second TwoSum before the small terms are added.
// Two outputs at once: packed float32x2 additions (IEEE round-to-nearest,
// each lane exactly the scalar operation).
__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, f2neg(a));
  e = __fadd2_rn(__fadd2_rn(a, f2neg(__fadd2_rn(s, f2neg(bb)))), __fadd2_rn(b, f2neg(bb)));
}
__device__ __forceinline__ void diag_pair2(const float2 (&a)[kDig], float2& H, float2& Lo) {
  float2 h, l, e, f, l2, e2;
  two_sum2(a[0], a[1], h, l);
  two_sum2(__fadd2_rn(l, a[2]), a[3], l2, e);
  two_sum2(__fadd2_rn(e, a[4]), a[5], e2, f);
  f = __fadd2_rn(f, a[6]);
  float2 s, t, t2;
  two_sum2(h, l2, s, t);
  two_sum2(s, e2, s, t2);
  two_sum2(s, __fadd2_rn(__fadd2_rn(t, t2), f), H, Lo);
}
// (H + Lo) 2^sh as a float64, from the bits with integer operations only
// (GB300's float64 pipe runs at 1/64 of the float32 rate).  With
// |Lo| <= ulp(H) / 2 the sum has H's exponent (or one less) and its
// significand is H's 24 bits followed by Lo's bits, rounded at 2^-52 of H
// (to nearest, ties up): error <= 2^-53 relative, as a float64 addition.
// Results below float64's normal range flush to zero (the caller's values
// are normalised per column, so these are ~2^-1000 of the column's largest).
__device__ __forceinline__ double pair_to_f64(float H, float Lo, int sh) {
  const unsigned hb = __float_as_uint(H);
  const int eh = (int)((hb >> 23) & 255);
  if (eh == 0) return 0.0;   // zero, or a float32 subnormal (< 2^-126 of the column scale)
  long long M = (long long)((hb & 0x7FFFFFu) | 0x800000u) << 29;   // 2^52 <= M < 2^53
  const unsigned lb = __float_as_uint(Lo);
  const int el = (int)((lb >> 23) & 255);
  if (el != 0) {
    const long long ml = (long long)((lb & 0x7FFFFFu) | 0x800000u);
    const int d = eh - el;   // >= 24
    long long add = 0;
    if (d <= 29) add = ml << (29 - d);
    else if (d < 54) add = (ml + (1LL << (d - 30))) >> (d - 29);
    M += ((hb ^ lb) >> 31) ? -add : add;
  }
  int e = eh - 127 + 1023 + sh;   // biased float64 exponent
  if (M < (1LL << 52)) {
    M <<= 1;
    e -= 1;
  }
  const unsigned long long sgn = (unsigned long long)(hb >> 31) << 63;
  if (e <= 0) return __longlong_as_double((long long)sgn);
  if (e >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double(
      (long long)(sgn | ((unsigned long long)e << 52) | ((unsigned long long)M & 0xFFFFFFFFFFFFFull)));
}

// ---------------------------------------------------------------- the kernel
// Tile t of a step: block b, row tile rt, column tile ct (ct fastest, so the
// consecutive tiles of a CTA share their operator digits).
struct Tile {
  int b, rt, ct;
};
__device__ __forceinline__ Tile tile_of(int t, int ntile, int nct) {
  Tile T;
  const int per_b = ntile * nct;
  T.b = t / per_b;
  const int rem = t - T.b * per_b;
  T.rt = rem / nct;
  T.ct = rem - T.rt * nct;
  return T;
}

// Persistent, warp-specialised: each CTA (one per SM) runs a contiguous range
// of tiles.  Digitiser warps (16) prepare tile i + 1 -- input rows, column
// scales, digit chunks -- while the MMA warp and the epilogue warps (8, two
// per TMEM lane quadrant) finish tile i; the accumulators of one tile fill
// the tensor memory, so the MMAs of tile i + 1 start when the epilogue has
// read tile i's.  mbarriers: op_full (operator digits landed), tmem_full
// (a tile's MMAs done), tmem_empty (its accumulators read), zfull / zempty
// (digit chunk buffers), cs_full / cs_free (column scales, by tile parity).
__global__ void __launch_bounds__(kThreads, 1) oz_step_kernel(const OzStep o) {
  extern __shared__ unsigned char smraw[];
  __shared__ __align__(8) uint64_t op_full, tmem_full, tmem_empty;
  __shared__ __align__(8) uint64_t zfull[2], zempty[2], cs_full[2], cs_free[2];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int s_fail;
  // per-role failure flags, written before and read after a role barrier so
  // every warp of the role takes the same branch (named barriers have no
  // timeout: a role must never leave its loop partly)
  __shared__ volatile int d_fail, e_fail;
  __shared__ const char* rowp[kMaxW];
  __shared__ int rowf64[kMaxW];
  __shared__ char* outp[kMaxNT];
  __shared__ const char* resp[kMaxNT];
  __shared__ int outf64[kMaxNT];
  __shared__ float rs[kMaxNT];
  __shared__ float colmax[kDigWarps / 4][kM];
  __shared__ float cscale[2][kM];

  const sweep::Step<dfloat>& s = o.s;
  const int NT = o.NT, wP = o.wP, w = s.w;
  const int nct = (s.c + kM - 1) / kM;
  const int ntiles = s.nb * o.ntile * nct;
  const int t0 = (int)((long long)blockIdx.x * ntiles / gridDim.x);
  const int nt = (int)((long long)(blockIdx.x + 1) * ntiles / gridDim.x) - t0;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t zsl = (uint32_t)kM * kKC * 2;   // one digit of one z chunk
  const uint32_t zdb = (uint32_t)kDig * zsl;     // one z chunk buffer (all digits)
  const uint32_t obytes = (uint32_t)NT * wP * 2; // one operator digit image
  const int nch = (wP + kKC - 1) / kKC;
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* zbuf = sm;             // two z chunk buffers
  unsigned char* opb = sm + 2 * zdb;    // the seven operator digit images
  uint32_t ncols = 32;
  while (ncols < (uint32_t)(kDig * NT)) ncols <<= 1;

  if (tid == 0) {
    mbar_init(&op_full, 1);
    mbar_init(&tmem_full, 1);
    mbar_init(&tmem_empty, kEpiWarps);
    for (int i = 0; i < 2; ++i) {
      mbar_init(&zfull[i], kDigWarps);
      mbar_init(&zempty[i], 1);
      mbar_init(&cs_full[i], kDigWarps);
      mbar_init(&cs_free[i], kEpiWarps);
    }
    s_fail = 0;
    d_fail = 0;
    e_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // the first tile's operator digits are constant: their copy starts before
  // the wait for the previous launch; the accumulators are allocated there
  // too (only a CTA still running on this SM can hold tensor memory, and it
  // frees it without waiting on this one)
  if (warp == kMmaWarp) {
    if (lane == 0 && nt > 0) {
      const Tile T = tile_of(t0, o.ntile, nct);
      mbar_expect_tx(&op_full, kDig * obytes);
      bulk_copy(opb, o.dig + (size_t)(T.b * o.ntile + T.rt) * kDig * NT * wP, kDig * obytes,
                &op_full);
    }
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  sweep::grid_dependency_wait();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == kMmaWarp) {
    // ---------------- MMA warp: digit pair (s, t), s + t <= 8 -> accumulator
    // s + t, chunk by chunk of z as the digitisers finish them
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NT >> 3) << 17) |
                             ((uint32_t)(kM >> 4) << 24);
      const uint32_t osbo = (uint32_t)wP * 16;   // operator: bytes per 8-row group
      const uint64_t ostep = obytes >> 4;
      bool fail = false;
      int g = 0, nload = 1;
      int opkey = -1;
      if (nt > 0) {
        const Tile T = tile_of(t0, o.ntile, nct);
        opkey = T.b * o.ntile + T.rt;
      }
      for (int i = 0; i < nt && !fail; ++i) {
        const Tile T = tile_of(t0 + i, o.ntile, nct);
        const int key = T.b * o.ntile + T.rt;
        if (key != opkey) {
          // new operator digits once the previous tile's MMAs have read the old
          if (!mbar_wait(&tmem_full, (uint32_t)((i - 1) & 1))) {
            fail = true;
            break;
          }
          mbar_expect_tx(&op_full, kDig * obytes);
          bulk_copy(opb, o.dig + (size_t)key * kDig * NT * wP, kDig * obytes, &op_full);
          opkey = key;
          ++nload;
        }
        if (!mbar_wait(&op_full, (uint32_t)((nload - 1) & 1))) {
          fail = true;
          break;
        }
        // the epilogue has read the previous tile's accumulators
        if (i > 0 && !mbar_wait(&tmem_empty, (uint32_t)((i - 1) & 1))) {
          fail = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int c = 0; c < nch; ++c, ++g) {
          const int b2 = g & 1;
          if (!mbar_wait(&zfull[b2], (uint32_t)(g >> 1) & 1u)) {
            fail = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const int ksteps = min(kKC, wP - c * kKC) / 16;
          // descriptors of digit 0 of the chunk (z) and of the operator at
          // this chunk's k; a start-address offset is added in 16-byte units
          const uint64_t a0 = desc_noswz(smem_u32(zbuf + b2 * zdb), 128, kKC * 16);
          const uint64_t b0 =
              desc_noswz(smem_u32(opb) + (uint32_t)c * (kKC / 8) * 128, 128, osbo);
          // every diagonal is first written by the pair (0, d) of the tile's
          // first k step: that MMA overwrites, every other one accumulates
#pragma unroll
          for (int si = 0; si < kDig; ++si) {
#pragma unroll
            for (int ti = 0; si + ti < kDig; ++ti) {
              const uint32_t dt = tmem + (uint32_t)((si + ti) * NT);
              const uint64_t ad = a0 + (uint64_t)((ti * zsl) >> 4);
              const uint64_t bd = b0 + (uint64_t)si * ostep;
              mma_bf16(dt, ad, bd, idesc, (c | si) != 0 ? 1u : 0u);
              if (ksteps > 1) mma_bf16(dt, ad + 16, bd + 16, idesc, 1u);
            }
          }
          mma_commit(&zempty[b2]);   // this chunk buffer is free once these MMAs finish
        }
        if (fail) break;
        mma_commit(&tmem_full);
      }
      if (fail) {
        s_fail = 1;
        if (o.err) atomicOr(o.err, 1u);
        __threadfence_block();
        // the last operator copy must land before the CTA exits
        mbar_wait(&op_full, (uint32_t)((nload - 1) & 1));
      }
    }
    __syncwarp();
  } else if (warp >= kDigWarps) {
    // ---------------- epilogue warps: warp (qd, rh) reads TMEM lanes 32 qd ..
    // (its columns) and the 8-row groups rh * 8 + 16 i of the tile
    const int qd = warp & 3, rh = (warp - kDigWarps) >> 2, etid = tid - kDigWarps * 32;
    const int col = qd * 32 + lane;
    const uint32_t lanes = (uint32_t)(qd * 32) << 16;
    for (int i = 0; i < nt; ++i) {
      const Tile T = tile_of(t0 + i, o.ntile, nct);
      const int c0 = T.ct * kM, r0 = T.rt * NT;
      const int nr = min(NT, s.rows - r0);
      // output row of every tile row, row scales (the previous tile's
      // readers are done: all four warps passed the barrier below)
      if (etid == 0 && s_fail) e_fail = 1;
      asm volatile("bar.sync 2, %0;" ::"r"(kEpiWarps * 32) : "memory");
      if (e_fail) continue;   // the same for every epilogue warp
      for (int r = etid; r < NT; r += kEpiWarps * 32) {
        char* p = nullptr;
        const char* pb = nullptr;
        int f = 0;
        float sc = 0.f;
        if (r < nr) {
          const int row = r0 + r;
          if (row < s.split) {
            const long long q = (long long)T.b * s.out_blk[0] + row;
            const long long dst = s.out_perm ? __ldg(s.out_perm + q) : q;
            p = reinterpret_cast<char*>(s.out_p[0] + dst * s.out_ld[0] + c0);
            f = o.out_f64;
            if (o.resb) pb = reinterpret_cast<const char*>(o.resb + dst * s.out_ld[0] + c0);
          } else {
            const long long q = (long long)T.b * s.out_blk[1] + (row - s.split);
            p = reinterpret_cast<char*>(s.out_p[1] + q * s.out_ld[1] + c0);
          }
          sc = __ldg(o.rsc + (size_t)(T.b * o.ntile + T.rt) * NT + r);
        }
        outp[r] = p;
        resp[r] = pb;
        outf64[r] = f;
        rs[r] = sc;
      }
      asm volatile("bar.sync 2, %0;" ::"r"(kEpiWarps * 32) : "memory");
      const bool ok = mbar_wait(&cs_full[i & 1], (uint32_t)((i >> 1) & 1)) &&
                      mbar_wait(&tmem_full, (uint32_t)(i & 1));
      __syncwarp();
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) {
          e_fail = 1;
          s_fail = 1;
          if (o.err) atomicOr(o.err, 1u);
        }
        continue;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const bool cok = c0 + col < s.c;
      // float64 outputs leave scaled back by 2^s_col
      const int osh = (o.colbits && cok) ? col_shift(__ldg(o.colbits + c0 + col)) : 0;
      const float csc = cscale[i & 1][col];
      float rsq = 0.f;   // squared residual norm of this column (residual form)
      for (int r8 = rh * 8; r8 < NT; r8 += 16) {
        uint32_t v[kDig][8];
        float hp[2], lp[2];
#pragma unroll
        for (int di = 0; di < kDig; ++di)
          tmem_ld8(tmem + lanes + (uint32_t)(di * NT + r8), v[di]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i8 = 0; i8 < 8; ++i8) {
          const int row = r8 + i8;
          // rows i8, i8 + 1 combined together (packed float32x2)
          float2 H2, L2;
          if ((i8 & 1) == 0) {
            float2 a[kDig];
#pragma unroll
            for (int di = 0; di < kDig; ++di)
              a[di] = make_float2(__uint_as_float(v[di][i8]), __uint_as_float(v[di][i8 + 1]));
            diag_pair2(a, H2, L2);
            hp[0] = H2.x;
            hp[1] = H2.y;
            lp[0] = L2.x;
            lp[1] = L2.y;
          }
          if (row >= nr || !cok) continue;
          float H = hp[i8 & 1], Lo = lp[i8 & 1];
          const float gs = __fmul_rn(rs[row], csc);   // a power of two, or 0
          char* p = outp[row] + 8 * col;
          if (outf64[row]) {
            const int ge = (int)((__float_as_uint(gs) >> 23) & 255);
            if (resp[row]) {
              // r = b - S z in the row's scale 2^sh: b split into a float
              // pair there (integer operations), one double-float
              // subtraction, then back to float64 like the plain output
              const int sh = ge ? ge - 127 + osh : osh;
              const double bv = *reinterpret_cast<const double*>(resp[row] + 8 * col);
              float bh, bl;
              f64_split(bv, sh, bh, bl);
              if (!ge) {
                H = 0.f;
                Lo = 0.f;
              }
              float rh, rl;
              two_sum(bh, -H, rh, rl);
              rl = __fadd_rn(rl, __fsub_rn(bl, Lo));
              two_sum(rh, rl, rh, rl);
              *reinterpret_cast<double*>(p) = pair_to_f64(rh, rl, sh);
              const float rr = ge ? __fmul_rn(rh, gs) : rh;
              rsq = __fmaf_rn(rr, rr, rsq);
            } else {
              *reinterpret_cast<double*>(p) = ge ? pair_to_f64(H, Lo, ge - 127 + osh) : 0.0;
            }
          } else {
            *reinterpret_cast<float2*>(p) = make_float2(__fmul_rn(H, gs), __fmul_rn(Lo, gs));
          }
        }
      }
      // the accumulators and this tile's column scales may be reused
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&tmem_empty);
        mbar_arrive(&cs_free[i & 1]);
      }
      // rsq holds the column's squares scaled by 2^(-2 osh)
      if (o.rnorm2 && cok && rsq > 0.f)
        atomicAdd(o.rnorm2 + c0 + col, ldexp((double)rsq, 2 * osh));
    }
  } else {
    // ---------------- digitiser warps (512 threads): thread (j, qk) owns
    // column j and the k of each chunk's quarter qk (8 k: one core-matrix row)
    const int j = tid & (kM - 1), qk = tid >> 7;
    int g = 0;
    bool fail = false;
    for (int i = 0; i < nt; ++i) {
      const Tile T = tile_of(t0 + i, o.ntile, nct);
      const int c0 = T.ct * kM;
      // input row of every k (the first range optionally through the
      // permutation); the previous tile's readers are done at this barrier
      if (fail) d_fail = 1;
      if (tid == 0 && s_fail) d_fail = 1;
      asm volatile("bar.sync 1, %0;" ::"r"(kDigWarps * 32) : "memory");
      if (d_fail) continue;   // the same for every digitiser warp
      for (int k = tid; k < w; k += kDigWarps * 32) {
        int q = 0, kk = k;
        while (q + 1 < s.nin && kk >= s.in_rows[q]) kk -= s.in_rows[q++];
        long long row = (long long)T.b * s.in_blk[q] + kk;
        if (q == 0 && s.in_perm) row = __ldg(s.in_perm + row);
        rowp[k] = reinterpret_cast<const char*>(s.in_p[q] + row * s.in_ld[q] + c0);
        rowf64[k] = (q == 0 && o.in_f64) ? 1 : 0;
      }
      asm volatile("bar.sync 1, %0;" ::"r"(kDigWarps * 32) : "memory");
      const bool col_ok = c0 + j < s.c;
      const int csh = (o.colbits && col_ok) ? col_shift(__ldg(o.colbits + c0 + j)) : 0;
      auto load = [&](int k, float& h, float& l) {
        h = 0.f;
        l = 0.f;
        if (col_ok && k < w) {
          const char* p = rowp[k] + 8 * j;
          if (rowf64[k]) {
            f64_split(*reinterpret_cast<const double*>(p), csh, h, l);
          } else {
            const float2 v = *reinterpret_cast<const float2*>(p);
            h = v.x;
            l = v.y;
          }
        }
      };
      // column scale: largest |h| over the column's k (8 loads in flight),
      // chunks in reverse order so that chunk 0's values stay in registers
      // for the first digitisation
      // (the next chunk's loads are in flight while this chunk is scanned)
      float mx = 0.f;
      float hv[8], lv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) hv[u] = lv[u] = 0.f;
      if ((nch - 1) * kKC + qk * 8 < wP) {
#pragma unroll
        for (int u = 0; u < 8; ++u) load((nch - 1) * kKC + qk * 8 + u, hv[u], lv[u]);
      }
      for (int c = nch - 1; c >= 0; --c) {
        float ph[8], pl[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) ph[u] = pl[u] = 0.f;
        if (c > 0 && (c - 1) * kKC + qk * 8 < wP) {
#pragma unroll
          for (int u = 0; u < 8; ++u) load((c - 1) * kKC + qk * 8 + u, ph[u], pl[u]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) mx = fmaxf(mx, fabsf(hv[u]));
        if (c > 0) {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            hv[u] = ph[u];
            lv[u] = pl[u];
          }
        }
      }
      colmax[qk][j] = mx;
      asm volatile("bar.sync 1, %0;" ::"r"(kDigWarps * 32) : "memory");
      float inv = 1.f, cs = 0.f;   // 2^-F and 2^F of the column (0: zero column)
      {
        const float m =
            fmaxf(fmaxf(colmax[0][j], colmax[1][j]), fmaxf(colmax[2][j], colmax[3][j]));
        if (m > 0.f) {
          // m < 2^(F - 1): the scaled column lies below 1/2, so every
          // digit is at most 128 units (256 for the fourth)
          int F = (int)((__float_as_uint(m) >> 23) & 255) - 125;
          F = max(-100, min(100, F));
          inv = __uint_as_float((unsigned)(127 - F) << 23);
          cs = __uint_as_float((unsigned)(127 + F) << 23);
        }
      }
      // publish the column scales for the epilogue (its tile i - 2 is done)
      if (i >= 2 && !mbar_wait(&cs_free[i & 1], (uint32_t)(((i >> 1) - 1) & 1))) fail = true;
      if (qk == 0) cscale[i & 1][j] = cs;
      __syncwarp();
      if (lane == 0) mbar_arrive(&cs_full[i & 1]);
      for (int c = 0; c < nch; ++c, ++g) {
        const int b2 = g & 1;
        const int k0 = c * kKC + qk * 8;
        // the next chunk's loads go out before this chunk is digitised
        float nh[8], nl[8];
        const bool more = c + 1 < nch && k0 + kKC < wP;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          nh[u] = 0.f;
          nl[u] = 0.f;
        }
        if (more) {
#pragma unroll
          for (int u = 0; u < 8; ++u) load(k0 + kKC + u, nh[u], nl[u]);
        }
        if (g >= 2 && !mbar_wait(&zempty[b2], (uint32_t)((g >> 1) - 1) & 1u)) fail = true;
        if (k0 < wP) {
          uint32_t wd[kDig][4];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            float hs = __fmul_rn(hv[u], inv), ls = __fmul_rn(lv[u], inv);
            float q[kDig];
            q[0] = extract(hs, 0x1.8p15f);
            hs = __fsub_rn(hs, q[0]);
            q[1] = extract(hs, 0x1.8p7f);
            hs = __fsub_rn(hs, q[1]);
            q[2] = extract(hs, 0x1.8p-1f);
            hs = __fsub_rn(hs, q[2]);
            float a, e;
            two_sum(hs, ls, a, e);
            q[3] = extract(a, 0x1.8p-9f);
            a = __fsub_rn(a, q[3]);
            q[4] = extract(a, 0x1.8p-17f);
            a = __fsub_rn(a, q[4]);
            float a2, e2;
            two_sum(a, e, a2, e2);
            q[5] = extract(a2, 0x1.8p-25f);
            a2 = __fsub_rn(a2, q[5]);
            q[6] = extract(__fadd_rn(a2, e2), 0x1.8p-33f);
            // two bfloat16 halves per word: the high halves of the float32
            // digits of k = u - 1 and u (one byte permute per pair)
            if (u & 1) {
#pragma unroll
              for (int t = 0; t < kDig; ++t)
                wd[t][u >> 1] = __byte_perm(wd[t][u >> 1], __float_as_uint(q[t]), 0x7632);
            } else {
#pragma unroll
              for (int t = 0; t < kDig; ++t) wd[t][u >> 1] = __float_as_uint(q[t]);
            }
          }
          // 16-byte row (8 k) of column j in core matrix (j / 8, qk)
          const uint32_t off = (uint32_t)(j >> 3) * (kKC * 16) + (uint32_t)qk * 128 +
                               (uint32_t)(j & 7) * 16;
          unsigned char* zb = zbuf + b2 * zdb + off;
#pragma unroll
          for (int t = 0; t < kDig; ++t)
            *reinterpret_cast<uint4*>(zb + (size_t)t * zsl) =
                make_uint4(wd[t][0], wd[t][1], wd[t][2], wd[t][3]);
        }
        // generic-proxy writes -> visible to the tensor cores; one arrival per warp
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&zfull[b2]);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          hv[u] = nh[u];
          lv[u] = nl[u];
        }
      }
    }
    sweep::launch_dependents();
    if (fail) {
      s_fail = 1;
      if (o.err) atomicOr(o.err, 1u);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
                 : "memory");
}

// ---------------------------------------------------------------- operator digits
// One warp per (block, row): the row's power-of-two scale and its seven
// balanced base-256 digits, written into the core-matrix images.
__global__ void oz_digits_kernel(const double* __restrict__ S, long long sS, int ld, int Nb,
                                 int rows, int w, int NT, int wP, int ntile,
                                 uint16_t* __restrict__ dig, float* __restrict__ rsc) {
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= Nb * rows) return;
  const int b = gw / rows, r = gw - b * rows;
  const double* row = S + (long long)b * sS + (long long)r * ld;
  double mx = 0.0;
  for (int k = lane; k < w; k += 32) mx = fmax(mx, fabs(row[k]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int E = 0;
  if (mx > 0.0) frexp(mx, &E);   // mx < 2^E
  E = max(-119, min(126, E)) + 1;   // rows scaled below 1/2: every digit <= 128
  const int rt = r / NT, rr = r - rt * NT;
  if (lane == 0) rsc[(size_t)(b * ntile + rt) * NT + rr] = mx > 0.0 ? ldexpf(1.f, E) : 0.f;
  if (mx == 0.0) return;
  uint16_t* img = dig + (size_t)(b * ntile + rt) * kDig * NT * wP;
  const size_t base = (size_t)(rr >> 3) * (wP * 8) + (size_t)(rr & 7) * 8;
  for (int k = lane; k < w; k += 32) {
    long long F = llrint(ldexp(row[k], 56 - E));   // |F| < 2^55
    int d[kDig];
    for (int t = kDig - 1; t >= 1; --t) {
      const long long dd = ((F + 128) & 255) - 128;
      d[t] = (int)dd;
      F = (F - dd) >> 8;
    }
    d[0] = (int)F;
    const size_t off = base + (size_t)(k >> 3) * 64 + (k & 7);
    for (int t = 0; t < kDig; ++t) {
      const float q = ldexpf((float)d[t], -8 * (t + 1));
      img[(size_t)t * NT * wP + off] = (uint16_t)(__float_as_uint(q) >> 16);
    }
  }
}

// colbits[j] = high word of the float64 bits of max_i |x_ij| (positive
// float64 bit patterns order like their values, so an integer atomicMax on
// the high words finds the largest exponent).  colbits must be zeroed first.
__global__ void oz_colmax_kernel(int rows, int c, const double* __restrict__ X, int ldx,
                                 unsigned* __restrict__ colbits) {
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  if (j >= c) return;
  unsigned m = 0;
  for (long long i = (long long)blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5); i < rows;
       i += (long long)gridDim.y * (blockDim.x >> 5)) {
    const unsigned hi = (unsigned)((unsigned long long)__double_as_longlong(X[i * ldx + j]) >> 32);
    m = max(m, hi & 0x7FFFFFFFu);
  }
  if (m) atomicMax(colbits + j, m);
}

void col_max(cudaStream_t st, int rows, int c, const double* X, int ldx, unsigned* colbits) {
  SLU_CHECK_CUDA(cudaMemsetAsync(colbits, 0, 4 * (size_t)c, st));
  dim3 grid((c + 31) / 32, (unsigned)std::min<long long>(64, std::max(1, rows / 64)));
  oz_colmax_kernel<<<grid, 256, 0, st>>>(rows, c, X, ldx, colbits);
  check_launch("oz_colmax_kernel");
}

void make_op(cudaStream_t st, OzOp& o, const double* S, int Nb, int rows, int w) {
  SLU_REQUIRE(S, "tensor-core sweep: step operator not composed");
  SLU_REQUIRE(w >= 1 && w <= kMaxW,
              "tensor-core sweep: a step reads " + std::to_string(w) +
                  " rows per block; at most 128 keep its digit sums exact");
  o.Nb = Nb;
  o.rows = rows;
  o.w = w;
  o.NT = rows > 32 ? 64 : (rows > 16 ? 32 : 16);
  // steps wider than 96: 32-row tiles keep the seven operator digit images
  // of a tile (NT x wP each) and the two z chunk buffers within 227 KB
  if (w > 96) o.NT = std::min(o.NT, 32);
  o.ntile = (rows + o.NT - 1) / o.NT;
  o.wP = (w + 15) / 16 * 16;
  const size_t nd = (size_t)Nb * o.ntile * kDig * o.NT * o.wP;
  o.dig.alloc(2 * nd, st);
  SLU_CHECK_CUDA(cudaMemsetAsync(o.dig.p, 0, 2 * nd, st));
  const size_t nr = (size_t)Nb * o.ntile * o.NT;
  o.rsc.alloc(4 * nr, st);
  SLU_CHECK_CUDA(cudaMemsetAsync(o.rsc.p, 0, 4 * nr, st));
  const long long warps = (long long)Nb * rows;
  oz_digits_kernel<<<(unsigned)((warps + 7) / 8), 256, 0, st>>>(
      S, (long long)rows * w, w, Nb, rows, w, o.NT, o.wP, o.ntile, o.dig.as<uint16_t>(),
      o.rsc.as<float>());
  check_launch("oz_digits_kernel");
}

void launch(cudaStream_t st, const sweep::Step<dfloat>& s, const OzOp& op, bool in_f64,
            bool out_f64, const unsigned* colbits, unsigned* err, const char* what,
            const double* resb = nullptr, double* rnorm2 = nullptr) {
  SLU_REQUIRE(op.dig.p && s.rows == op.rows && s.w == op.w && s.nb == op.Nb,
              "tensor-core sweep: digit operator does not match its step");
  OzStep o{};
  o.s = s;
  o.dig = op.dig.as<uint16_t>();
  o.rsc = op.rsc.as<float>();
  o.NT = op.NT;
  o.wP = op.wP;
  o.ntile = op.ntile;
  o.in_f64 = in_f64 ? 1 : 0;
  o.out_f64 = out_f64 ? 1 : 0;
  o.colbits = (in_f64 || out_f64) ? colbits : nullptr;
  o.err = err;
  SLU_REQUIRE(!resb || (out_f64 && s.out_ld[0] >= s.c), "residual form needs a float64 output");
  o.resb = resb;
  o.rnorm2 = rnorm2;
  sweep::LaunchPlan p;
  const long long ntiles = (long long)s.nb * op.ntile * ((s.c + kM - 1) / kM);
  p.ctas = std::min<long long>(ntiles, num_sms());   // persistent: one CTA per SM
  p.threads = kThreads;
  p.smem = smem_bytes(op.NT, op.wP);
  SLU_REQUIRE(ntiles < (1LL << 31), "tensor-core sweep: step too large");
  ensure_smem(reinterpret_cast<const void*>(oz_step_kernel), p.smem);
  sweep::launch_pdl(oz_step_kernel, p, st, what, o);
}

}  // namespace oz

void hbs_make_oz(Handle& h, Hbs& H) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed (factor the operator first)");
  std::lock_guard<std::mutex> lock(H.lazy_mu);
  if (H.has_oz) return;
  if (!H.has_apply[0]) hbs_make_apply(h, H, false);
  cudaStream_t st = h.stream;
  const int L = H.L;
  for (int t = 0; t + 1 < L; ++t) {
    Level& l = H.lv[t];
    oz::make_op(st, l.ozQt, l.Qt.as<double>(), l.Nb, l.n, l.n);
    oz::make_op(st, l.ozSw, l.Sw.as<double>(), l.Nb, t == 0 ? l.n : 2 * l.n, l.nu + 2 * l.k);
    oz::make_op(st, l.ozUp, l.Aup.as<double>(), l.Nb, l.k, l.n);
    oz::make_op(st, l.ozDn, l.Adn.as<double>(), l.Nb, l.n, l.n + l.k);
  }
  Level& r = H.lv[L - 1];
  oz::make_op(st, r.ozSw, r.Sw.as<double>(), 1, L == 1 ? r.n : 2 * r.n, r.n);
  oz::make_op(st, r.ozDn, r.Adn.as<double>(), 1, r.n, r.n);
  stream_wait(st);
  H.has_oz = true;
}

void hbs_make_ozT(Handle& h, Hbs& H) {
  SLU_REQUIRE(H.has_sweep, "step operators not composed (factor the operator first)");
  std::lock_guard<std::mutex> lock(H.lazy_mu);
  if (H.has_ozT) return;
  if (!H.has_apply[1]) hbs_make_apply(h, H, true);
  cudaStream_t st = h.stream;
  const int L = H.L;
  for (int t = 0; t + 1 < L; ++t) {
    Level& l = H.lv[t];
    oz::make_op(st, l.ozQ, l.Q.as<double>(), l.Nb, l.n, l.n);
    oz::make_op(st, l.ozSwT, l.SwT.as<double>(), l.Nb, l.nu + 2 * l.k, t == 0 ? l.n : 2 * l.n);
    oz::make_op(st, l.ozUpT, l.AupT.as<double>(), l.Nb, l.k, l.n);
    oz::make_op(st, l.ozDnT, l.AdnT.as<double>(), l.Nb, l.n, l.n + l.k);
  }
  Level& r = H.lv[L - 1];
  oz::make_op(st, r.ozSwT, r.SwT.as<double>(), 1, r.n, L == 1 ? r.n : 2 * r.n);
  oz::make_op(st, r.ozDnT, r.AdnT.as<double>(), 1, r.n, r.n);
  stream_wait(st);
  H.has_ozT = true;
}

size_t hbs_oz_scratch_bytes(const Hbs& H, int c) {
  const size_t nc = ((size_t)H.N * c + 63) & ~size_t(63);
  const size_t solve = 5 * nc;
  const size_t apply = hbs_apply_scratch_elems(H, c);
  return sizeof(dfloat) * std::max(solve, apply) + (((size_t)4 * c + 255) & ~size_t(255)) + 256;
}

namespace {
// Scratch split: the column maxima first, the step vectors after them.
unsigned* oz_colbits(void* scratch) { return static_cast<unsigned*>(scratch); }
dfloat* oz_vectors(void* scratch, int c) {
  return reinterpret_cast<dfloat*>(static_cast<char*>(scratch) +
                                   (((size_t)4 * c + 255) & ~size_t(255)));
}
}  // namespace

void ulv_solve_oz(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch, unsigned* err) {
  SLU_REQUIRE(H.has_oz, "tensor-core sweep not prepared");
  SLU_REQUIRE(static_cast<const void*>(X) != static_cast<const void*>(Y),
              "tensor-core sweep: input and output must be different buffers");
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  const size_t nc = ((size_t)H.N * c + 63) & ~size_t(63);
  unsigned* cb = oz_colbits(scratch);
  dfloat* ws = oz_vectors(scratch, c);
  dfloat* ru = ws;
  dfloat* P[4] = {ws + nc, ws + 2 * nc, ws + 3 * nc, ws + 4 * nc};
  // the caller's float64 vectors are read by the first step and written by
  // the last; the step vectors in between are double-float pairs
  const dfloat* x = reinterpret_cast<const dfloat*>(X);
  dfloat* y = reinterpret_cast<dfloat*>(Y);
  const std::vector<long long>& NN = H.NN;
  oz::col_max(st, H.N, c, X, ldx, cb);
  if (L == 1) {
    sweep::Step<dfloat> s = sweep::root_step<dfloat>(H, x, ldx, y, ldy, nullptr, nullptr, c);
    s.in_p[0] = x;
    s.in_ld[0] = ldx;
    oz::launch(st, s, H.lv[0].ozSw, true, true, cb, err, "oz_root_step");
    return;
  }
  const dfloat* src = x;
  int lds = ldx;
  for (int t = 0; t + 1 < L; ++t) {
    oz::launch(st,
               sweep::forward_step<dfloat>(H, t, src, lds, t == 0 ? perm : nullptr,
                                           ru + NN[t] * c, P[t & 1], c),
               H.lv[t].ozQt, t == 0, false, cb, err, "oz_fwd_step");
    src = P[t & 1];
    lds = c;
  }
  oz::launch(st, sweep::root_step<dfloat>(H, src, lds, y, ldy, P[2], P[3], c), H.lv[L - 1].ozSw,
             false, false, cb, err, "oz_root_step");
  int in = 2;
  for (int t = L - 2; t >= 0; --t) {
    const int out = (in == 2) ? 0 : 2;
    oz::launch(st,
               sweep::backward_step<dfloat>(H, t, ru + NN[t] * c, P[in + 1], P[in], P[out],
                                            P[out + 1], y, ldy, c),
               H.lv[t].ozSw, false, t == 0, cb, err, "oz_bwd_step");
    in = out;
  }
}

// The transposed steps of ulv_solve_T (ulv_solve.cu, solve_steps_T) on the
// tensor cores: backward^T steps up the tree (the caller's rows gathered
// through the inverse permutation), the root^T step, forward^T steps down
// (Q itself), the result scattered through the inverse permutation.
void ulv_solve_oz_T(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y,
                    int ldy, int c, void* scratch, unsigned* err) {
  SLU_REQUIRE(H.has_ozT, "tensor-core transposed sweep not prepared");
  SLU_REQUIRE(static_cast<const void*>(X) != static_cast<const void*>(Y),
              "tensor-core sweep: input and output must be different buffers");
  const int L = H.L;
  const int64_t* ip = H.iperm.as<int64_t>();
  const size_t nc = ((size_t)H.N * c + 63) & ~size_t(63);
  unsigned* cb = oz_colbits(scratch);
  dfloat* ws = oz_vectors(scratch, c);
  dfloat* ru = ws;
  dfloat* P[2] = {ws + nc, ws + 3 * nc};   // two strides each (a backward^T writes 2k rows)
  const dfloat* x = reinterpret_cast<const dfloat*>(X);
  dfloat* y = reinterpret_cast<dfloat*>(Y);
  const std::vector<long long>& NN = H.NN;
  oz::col_max(st, H.N, c, X, ldx, cb);
  if (L == 1) {
    oz::launch(st, sweep::rootT_step<dfloat>(H, x, ldx, ip, y, ldy, ip, c), H.lv[0].ozSwT, true,
               true, cb, err, "oz_rootT_step");
    return;
  }
  for (int t = 0; t + 1 < L; ++t)
    oz::launch(st,
               sweep::backwardT_step<dfloat>(H, t, t == 0 ? x : P[(t - 1) & 1], t == 0 ? ldx : c,
                                             t == 0 ? ip : nullptr, ru + NN[t] * c, P[t & 1], c),
               H.lv[t].ozSwT, t == 0, false, cb, err, "oz_bwdT_step");
  int cur = (L - 1) & 1;
  oz::launch(st, sweep::rootT_step<dfloat>(H, P[(L - 2) & 1], c, nullptr, P[cur], c, nullptr, c),
             H.lv[L - 1].ozSwT, false, false, cb, err, "oz_rootT_step");
  for (int t = L - 2; t >= 0; --t) {
    const bool leaf = t == 0;
    oz::launch(st,
               sweep::forwardT_step<dfloat>(H, t, ru + NN[t] * c, P[cur], leaf ? y : P[cur ^ 1],
                                            leaf ? ldy : c, leaf ? ip : nullptr, c),
               H.lv[t].ozQ, false, leaf, cb, err, "oz_fwdT_step");
    cur ^= 1;
  }
}

void hbs_apply_oz(cudaStream_t st, const Hbs& H, const double* X, int ldx, double* Y, int ldy,
                  int c, void* scratch, unsigned* err, const double* resb, double* rnorm2,
                  bool trans) {
  SLU_REQUIRE(trans ? H.has_ozT : H.has_oz, "tensor-core apply not prepared");
  SLU_REQUIRE(static_cast<const void*>(X) != static_cast<const void*>(Y),
              "tensor-core apply: input and output must be different buffers");
  const int L = H.L;
  const int64_t* perm = H.perm.as<int64_t>();
  unsigned* cb = oz_colbits(scratch);
  dfloat* ws = oz_vectors(scratch, c);
  const dfloat* x = reinterpret_cast<const dfloat*>(X);
  dfloat* y = reinterpret_cast<dfloat*>(Y);
  std::vector<dfloat*> VV(L, nullptr);
  size_t off = 0;
  for (int t = 0; t + 1 < L; ++t) {
    VV[t + 1] = ws + off;
    off += ((size_t)H.lv[t].Nb * H.lv[t].k * c + 63) & ~size_t(63);
  }
  dfloat* u[2] = {ws + off, ws + off + (((size_t)H.N * c + 63) & ~size_t(63))};
  oz::col_max(st, H.N, c, X, ldx, cb);
  if (L == 1) {
    const Level& r = H.lv[0];
    oz::launch(st,
               sweep::down_step<dfloat>(r, nullptr, true, x, ldx, perm, nullptr, y, ldy, perm, c),
               (trans ? r.ozDnT : r.ozDn), true, true, cb, err, "oz_apply_root", resb, rnorm2);
    return;
  }
  for (int t = 0; t + 1 < L; ++t) {
    const Level& l = H.lv[t];
    oz::launch(st,
               sweep::up_step<dfloat>(l, nullptr, t == 0 ? x : VV[t], t == 0 ? ldx : c,
                                      t == 0 ? perm : nullptr, VV[t + 1], c),
               (trans ? l.ozUpT : l.ozUp), t == 0, false, cb, err, "oz_apply_up");
  }
  const Level& r = H.lv[L - 1];
  oz::launch(st,
             sweep::down_step<dfloat>(r, nullptr, true, VV[L - 1], c, nullptr, nullptr, u[0], c,
                                      nullptr, c),
             (trans ? r.ozDnT : r.ozDn), false, false, cb, err, "oz_apply_root");
  int cur = 0;
  for (int t = L - 2; t >= 0; --t) {
    const Level& l = H.lv[t];
    const bool leaf = t == 0;
    oz::launch(st,
               sweep::down_step<dfloat>(l, nullptr, false, leaf ? x : VV[t], leaf ? ldx : c,
                                        leaf ? perm : nullptr, u[cur], leaf ? y : u[cur ^ 1],
                                        leaf ? ldy : c, leaf ? perm : nullptr, c),
               (trans ? l.ozDnT : l.ozDn), leaf, leaf, cb, err, "oz_apply_down", leaf ? resb : nullptr,
               leaf ? rnorm2 : nullptr);
    cur ^= 1;
  }
}

}  // namespace slu
