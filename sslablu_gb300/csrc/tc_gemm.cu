// Tensor-core (tcgen05) GEMM for the dense contractions of the mixed-precision
// path: sketch products Y = S * Om of dense interface blocks (the sampling of
// matAssembly/matAssembler.py:112-117 and of the implicit Schur operators of
// direct_solve/omsdirectsolveHBS.py:57-179) and the Schur-complement products
// of the red-black elimination (direct_solve/omsdirectsolve.py:316-324).
//
// C (M x N, float64) = alpha * A (M x K, float64) * B (K x N, float64) + beta * C
// evaluated as a split-BF16x3 product: each float64 operand is split into
// three bfloat16 slices x = x0 + x1 + x2 (24 significant bits), and the six
// cross products x0y0 + x0y1 + x1y0 + x0y2 + x1y1 + x2y0 are accumulated by
// one tcgen05 GEMM over the concatenated K, in float32.  Relative accuracy is
// that of a float32 GEMM of depth 512, which is what the refinement-driven
// mixed path needs; the float64 path never uses this kernel.
//
// Kernel: one CTA per 128 x BN output tile (BN = 256 when the grid still
// fills the GPU, else 128), 320 threads, one CTA per SM; tiles in bands of
// 16 tile rows, column by column within a band (operand panels reused from
// L2 by the CTAs resident together).
//   warp 8 lane 0 : TMA producer, ring of (A 128 x 64, B BN x 64) bf16 slabs
//                   (128B-swizzled, one mbarrier per stage, complete_tx); the
//                   slice of each product is picked by the TMA coordinate
//   warp 9 lane 0 : MMA issuer, tcgen05.mma.cta_group::1.kind::f16
//                   (M=128, N=BN, K=16 per instruction) into two ping-pong
//                   float32 TMEM accumulators of BN columns; tcgen05.commit
//                   frees each stage and publishes each chunk; warp 9 also
//                   allocates and frees the 2 BN TMEM columns
//   warps 0-7     : epilogue; warp w reads TMEM lanes 32 (w % 4) .. + 31
//                   (its tile rows) and columns (w / 4) BN/2 .. + BN/2, adds
//                   each finished chunk into float32 sums (BN = 128: held in
//                   registers while the MMA fills the other accumulator;
//                   BN = 256: held in the second half of TMEM, the MMA waiting
//                   for each drain), stages the tile in the freed operand
//                   ring and writes C in float64, coalesced
// The product x0 y0 runs in chunks of 512 terms (1024 at BN = 256): float32
// rounding acts within a chunk; the float32 sums take ceil(K / 512) + 1 chunk
// additions.  The five smaller products (magnitudes <= 2^-8 of the result)
// form one last chunk.
// Every mbarrier wait is bounded; on timeout the kernel records an error word,
// drains what it issued (again bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "slablu_internal.cuh"

namespace slu {
namespace {

constexpr int BM = 128, BK = 64;
constexpr int A_BYTES = BM * BK * 2;             // 16 KB per A slab
constexpr int CHUNK = 8;                         // k-tiles (of BK) per x0 y0 chunk
constexpr int kEpiWarps = 8;
constexpr int kThreadsTC = 32 * (kEpiWarps + 2); // warps 0-7 epilogue, 8 TMA, 9 MMA
constexpr long long kWaitLimit = 1LL << 22;      // try_wait rounds before giving up
constexpr int kBand = 16;                        // tile rows per band of the tile order

template <int BN>
struct TcCfg {
  // BN = 128: two ping-pong accumulators, float32 sums in the epilogue's
  // registers.  BN = 256: one accumulator and the float32 sums in the other
  // half of TMEM (128 register sums per thread do not fit beside 10 warps);
  // the MMA waits for each drain, so chunks are twice as long.
  static constexpr bool kTmemSum = BN == 256;
  static constexpr int kChunk = kTmemSum ? 2 * CHUNK : CHUNK;
  static constexpr int kStages = BN == 256 ? 4 : 6;
  static constexpr int kStageBytes = A_BYTES + BN * BK * 2;
  static constexpr int kSmem = kStages * kStageBytes + 1024;   // + 1024 B alignment slack
  static constexpr uint32_t kTmemCols = 2 * BN;                // two accumulators
  static constexpr int kCols = BN / 2;                         // columns per epilogue thread
  // instruction descriptor, kind::f16: D f32, A/B bf16, both K-major, M = 128, N = BN
  static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                                     ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  static_assert(kSmem <= 227 * 1024, "shared memory");
  static_assert(BM * (BN + 1) * 4 <= kStages * kStageBytes, "epilogue staging fits the ring");
};

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

// Bounded wait for the phase with the given parity; returns false on timeout.
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

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128B swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);       // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused, swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset
  d |= (uint64_t)1 << 46;                        // descriptor version
  d |= (uint64_t)2 << 61;                        // SWIZZLE_128B
  return d;
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}

// Chunks of the K stream (k-tiles kt of KT = 6 KT1): the x0 y0 product
// (kt < KT1) in chunks of `chunk` k-tiles, the other five products as one.
__device__ __forceinline__ int chunk_count(int KT1, int chunk) {
  return (KT1 + chunk - 1) / chunk + 1;
}

// BN = 128: chunk c accumulates in float32 TMEM accumulator c % 2; the
// epilogue warps add each finished chunk into their register sums while the
// MMA warp fills the other accumulator.  BN = 256: every chunk uses the one
// accumulator, and the epilogue adds it into the TMEM sums before the next.
// (10 warps put 3 on some SM sub-partitions: 168 registers per thread at most)
template <int BN>
__global__ void __maxnreg__(168)
tc_gemm_bf16_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    int M, int N, int Kp, double alpha, double beta, double* __restrict__ C,
                    int ldc, unsigned int* __restrict__ err) {
  using G = TcCfg<BN>;
  constexpr int STAGES = G::kStages;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t ready_bar[2];
  __shared__ __align__(8) uint64_t drained_bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  __shared__ volatile int s_issued;   // TMA stages issued by the producer
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // grouped tile order: the tiles run in bands of kBand tile rows, column
  // by column inside a band, so the CTAs resident at one time share a few A
  // row panels and a few B column panels (row-major order re-read every B
  // panel once per few rows of tiles)
  int tm, tn;
  {
    const int tiles_n = (N + BN - 1) / BN, tiles_m = (M + BM - 1) / BM;
    const int id = blockIdx.x;
    const int band = id / (kBand * tiles_n);
    const int first = band * kBand;
    const int rows = min(tiles_m - first, kBand);
    const int in = id - band * kBand * tiles_n;
    tm = first + in % rows;
    tn = in / rows;
  }
  const int m0 = tm * BM, n0 = tn * BN;
  const int KT1 = Kp / BK;          // k-tiles of one product
  const int KT = 6 * KT1;
  const int NC = chunk_count(KT1, G::kChunk);

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&ready_bar[a], 1);
      mbar_init(&drained_bar[a], 32 * kEpiWarps);
    }
    s_fail = 0;
    s_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kEpiWarps + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(G::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == kEpiWarps) {
    // ---------------- TMA producer
    if (lane == 0) {
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % STAGES;
        if (kt >= STAGES && !mbar_wait(&empty_bar[s], ((kt / STAGES) + 1) & 1)) {
          s_fail = 1;
          break;
        }
        // product t = A slice sa x B slice sb: (0,0) (0,1) (1,0) (0,2) (1,1) (2,0)
        const int t = kt / KT1, kk = kt - t * KT1;
        const int sa = t == 0 ? 0 : (t == 1 ? 0 : (t == 2 ? 1 : (t == 3 ? 0 : (t == 4 ? 1 : 2))));
        const int sb = t == 0 ? 0 : (t == 1 ? 1 : (t == 2 ? 0 : (t == 3 ? 2 : (t == 4 ? 1 : 0))));
        unsigned char* a = smem + s * G::kStageBytes;
        unsigned char* b = a + A_BYTES;
        mbar_expect_tx(&full_bar[s], G::kStageBytes);
        tma_load_2d(a, &tmA, sa * Kp + kk * BK, m0, &full_bar[s]);
        tma_load_2d(b, &tmB, sb * Kp + kk * BK, n0, &full_bar[s]);
        s_issued = kt + 1;
      }
    }
  } else if (warp == kEpiWarps + 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      int kt = 0;
      bool fail = false;
      for (int c = 0; c < NC && !fail; ++c) {
        // accumulator of chunk c, and the drain it must wait for
        const int a = G::kTmemSum ? 0 : (c & 1);
        const bool reuse = G::kTmemSum ? c >= 1 : c >= 2;
        const uint32_t par = G::kTmemSum ? ((c - 1) & 1) : (((c >> 1) - 1) & 1);
        if (reuse && !mbar_wait(&drained_bar[a], par)) {
          fail = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(a * BN);
        const int kend = kt < KT1 ? min(kt + G::kChunk, KT1) : KT;
        for (int j = 0; kt < kend; ++j, ++kt) {
          const int s = kt % STAGES;
          if (!mbar_wait(&full_bar[s], (kt / STAGES) & 1)) {
            fail = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(smem + s * G::kStageBytes);
          const uint32_t sb = sa + A_BYTES;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16(dacc, smem_desc(sa + kk * 32), smem_desc(sb + kk * 32), G::kIdesc,
                     (j | kk) != 0);
          mma_commit(&empty_bar[s]);
        }
        mma_commit(&ready_bar[a]);
      }
      if (fail) {
        s_fail = 1;
        // let the copies already issued land before the CTA can exit
        const int issued = s_issued;
        for (int j = kt + 1; j < issued; ++j) mbar_wait(&full_bar[j % STAGES], (j / STAGES) & 1);
        mma_commit(&ready_bar[0]);
        mma_commit(&ready_bar[1]);
      }
    }
  } else {
    // ---------------- epilogue warps: TMEM lanes 32 (warp % 4) .., columns half (warp / 4)
    const int q = warp & 3, half = warp >> 2;
    const int r = q * 32 + lane;       // tile row owned by this thread
    constexpr int P = BN + 1;          // staging pitch (odd: no bank conflicts)
    float* tile = reinterpret_cast<float*>(smem);
    float run[G::kTmemSum ? 1 : G::kCols];
    if constexpr (!G::kTmemSum) {
#pragma unroll
      for (int j = 0; j < G::kCols; ++j) run[j] = 0.f;
    }
    bool fail = false;
    for (int c = 0; c < NC; ++c) {
      const int a = G::kTmemSum ? 0 : (c & 1);
      const uint32_t par = G::kTmemSum ? (c & 1) : ((c >> 1) & 1);
      // warp-uniform: the TMEM loads below are warp-collective
      const bool ok = mbar_wait(&ready_bar[a], par) && !s_fail;
      if (!__all_sync(0xffffffffu, ok)) {
        fail = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t lanes = (uint32_t)(q * 32) << 16;
      const uint32_t base = tmem + lanes + (uint32_t)(a * BN + half * G::kCols);
      if constexpr (G::kTmemSum) {
        // sums at columns BN ..: sum += chunk; the last chunk goes (with
        // the sums) straight to the staging tile, as every MMA has completed
        const uint32_t sbase = tmem + lanes + (uint32_t)(BN + half * G::kCols);
        const bool last = c == NC - 1;
#pragma unroll 1
        for (int c0 = 0; c0 < G::kCols; c0 += 32) {
          uint32_t v0[16], v1[16], u0[16], u1[16];
          tmem_ld16(base + (uint32_t)c0, v0);
          tmem_ld16(base + (uint32_t)c0 + 16, v1);
          if (c > 0) {
            tmem_ld16(sbase + (uint32_t)c0, u0);
            tmem_ld16(sbase + (uint32_t)c0 + 16, u1);
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float x0 = __uint_as_float(v0[j]), x1 = __uint_as_float(v1[j]);
            u0[j] = __float_as_uint(c > 0 ? __uint_as_float(u0[j]) + x0 : x0);
            u1[j] = __float_as_uint(c > 0 ? __uint_as_float(u1[j]) + x1 : x1);
          }
          if (!last) {
            tmem_st16(sbase + (uint32_t)c0, u0);
            tmem_st16(sbase + (uint32_t)c0 + 16, u1);
          } else {
            float* t = tile + r * P + half * G::kCols + c0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              t[j] = __uint_as_float(u0[j]);
              t[16 + j] = __uint_as_float(u1[j]);
            }
          }
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      } else {
#pragma unroll
        for (int c0 = 0; c0 < G::kCols; c0 += 16) {
          uint32_t v[16];
          tmem_ld16(base + (uint32_t)c0, v);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j) run[c0 + j] += __uint_as_float(v[j]);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&drained_bar[a]);
    }
    // one decision for all epilogue threads (each gave up, or not, on its
    // own bounded waits): they all pass this barrier, so the staging
    // barrier below is reached by all 256 or by none
    uint32_t any_fail;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.cta.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(any_fail)
        : "r"((uint32_t)fail), "r"(32 * kEpiWarps)
        : "memory");
    if (any_fail) {
      if (lane == 0 && err) atomicOr(err, 1u);
    } else {
      // every MMA has completed (the last chunk's commit), so the operand
      // ring is free: the sums are staged there (odd pitch: no bank
      // conflicts in either direction), then C is written row by row,
      // coalesced
      if constexpr (!G::kTmemSum) {
#pragma unroll
        for (int j = 0; j < G::kCols; ++j) tile[r * P + half * G::kCols + j] = run[j];
      }
      asm volatile("barrier.cta.sync 1, %0;" ::"r"(32 * kEpiWarps) : "memory");
      for (int e = threadIdx.x; e < BM * BN; e += 32 * kEpiWarps) {
        const int i = e / BN, j = e - i * BN;
        const int row = m0 + i, col = n0 + j;
        if (row < M && col < N) {
          double* cp = C + (long long)row * ldc + col;
          const double v = alpha * (double)tile[i * P + j];
          *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kEpiWarps + 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(G::kTmemCols)
                 : "memory");
}

// ---------------------------------------------------------------- splitting
// Slices of x: f = float32(x), s0 = bf16(f), s1 = bf16(f - s0),
// s2 = bf16(f - s0 - s1).  The differences are exact in float32 (each drops
// the leading 8 significant bits), so s0 + s1 + s2 carries the 24 bits of f:
// one float64 operation per element (GB300's float64 pipe is ~1/64 of the
// float32 one).
__device__ __forceinline__ void split3(double x, __nv_bfloat16& s0, __nv_bfloat16& s1,
                                       __nv_bfloat16& s2) {
  const float f = __double2float_rn(x);
  s0 = __float2bfloat16_rn(f);
  const float r1 = f - __bfloat162float(s0);
  s1 = __float2bfloat16_rn(r1);
  s2 = __float2bfloat16_rn(r1 - __bfloat162float(s1));
}

// A (M x K row-major, float64) -> Asl (M x 3*Kp bf16): slice t at columns
// t*Kp ..; one row per blockIdx.y, four consecutive k per thread (8-byte
// stores; Kp is a multiple of 64).
__global__ void split_a_kernel(int M, int K, int Kp, const double* __restrict__ A, int lda,
                               __nv_bfloat16* __restrict__ out) {
  const int i = blockIdx.y;
  const int k = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= M || k >= Kp) return;
  const double* a = A + (long long)i * lda;
  __align__(8) __nv_bfloat16 s[3][4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (k + u < K) split3(a[k + u], s[0][u], s[1][u], s[2][u]);
    else s[0][u] = s[1][u] = s[2][u] = __float2bfloat16_rn(0.f);
  }
  __nv_bfloat16* row = out + (long long)i * 3 * Kp + k;
#pragma unroll
  for (int t = 0; t < 3; ++t)
    *reinterpret_cast<uint2*>(row + (long long)t * Kp) = *reinterpret_cast<const uint2*>(s[t]);
}

// B (K x N row-major, float64) -> Bsl (N x 3*Kp bf16, K-major): slice t at
// columns t*Kp ..; 64 x 64 tiles transposed through shared memory (one
// float32 per element: the conversion happens on the way in).
__global__ void split_b_kernel(int K, int N, int Kp, const double* __restrict__ B, int ldb,
                               __nv_bfloat16* __restrict__ out) {
  __shared__ float tile[64][65];
  const int k0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;   // 256 threads: 64 x 4
  for (int r = ty; r < 64; r += 4) {
    const int k = k0 + r, n = n0 + tx;
    tile[r][tx] = (k < K && n < N) ? __double2float_rn(B[(long long)k * ldb + n]) : 0.f;
  }
  __syncthreads();
  // each thread: 4 consecutive k of one column n (8-byte stores)
  const int kq = 4 * (threadIdx.x & 15), nr = threadIdx.x >> 4;   // 16 x 16
  for (int c = nr; c < 64; c += 16) {
    const int n = n0 + c, k = k0 + kq;
    if (n >= N || k >= Kp) continue;
    __align__(8) __nv_bfloat16 s[3][4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float f = tile[kq + u][c];
      s[0][u] = __float2bfloat16_rn(f);
      const float r1 = f - __bfloat162float(s[0][u]);
      s[1][u] = __float2bfloat16_rn(r1);
      s[2][u] = __float2bfloat16_rn(r1 - __bfloat162float(s[1][u]));
    }
    __nv_bfloat16* row = out + (long long)n * 3 * Kp + k;
#pragma unroll
    for (int t = 0; t < 3; ++t)
      *reinterpret_cast<uint2*>(row + (long long)t * Kp) = *reinterpret_cast<const uint2*>(s[t]);
  }
}

// ---------------------------------------------------------------- host
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  if (!fn) throw Error(SLU_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  return fn;
}

// rows x cols bf16 matrix, row pitch cols (K-major), box 64 x box_rows, 128B swizzle.
CUtensorMap make_map(const void* base, int rows, long long cols, int box_rows) {
  SLU_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0, "TMA base must be 16-byte aligned");
  SLU_REQUIRE((cols * 2) % 16 == 0, "TMA row pitch must be a multiple of 16 bytes");
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(SLU_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return m;
}

template <int BN>
void launch_tc(cudaStream_t st, const __nv_bfloat16* Asl, const __nv_bfloat16* Bsl, int M, int N,
               int Kp, double alpha, double beta, double* C, int ldc, unsigned int* err) {
  using G = TcCfg<BN>;
  CUtensorMap ma = make_map(Asl, M, 3LL * Kp, BM);
  CUtensorMap mb = make_map(Bsl, N, 3LL * Kp, BN);
  ensure_smem(reinterpret_cast<const void*>(tc_gemm_bf16_kernel<BN>), G::kSmem);
  const long long tiles = (long long)((N + BN - 1) / BN) * ((M + BM - 1) / BM);
  SLU_REQUIRE(tiles < (1LL << 31), "GEMM has too many tiles");
  tc_gemm_bf16_kernel<BN><<<(unsigned)tiles, kThreadsTC, G::kSmem, st>>>(ma, mb, M, N, Kp, alpha,
                                                                          beta, C, ldc, err);
  check_launch("tc_gemm_bf16_kernel");
}

}  // namespace

size_t tc_gemm_workspace_bytes(int M, int N, int K) {
  const long long Kp = ((long long)K + BK - 1) / BK * BK;
  return (size_t)(3 * Kp * 2) * ((size_t)M + N) + 2 * 256;
}

// C = alpha A B + beta C with split-BF16x3 tcgen05 products (float32 accumulation).
// ws: tc_gemm_workspace_bytes(M, N, K) bytes; err: device word set on a wait timeout.
void tc_gemm_split3(cudaStream_t st, int M, int N, int K, double alpha, const double* A, int lda,
                    const double* B, int ldb, double beta, double* C, int ldc, void* ws,
                    unsigned int* err) {
  if (M <= 0 || N <= 0) return;
  SLU_REQUIRE(K >= 1, "K must be positive");
  const int Kp = (K + BK - 1) / BK * BK;
  SLU_REQUIRE(6LL * Kp < (1LL << 31), "K too large");
  __nv_bfloat16* Asl = reinterpret_cast<__nv_bfloat16*>(ws);
  size_t abytes = ((size_t)M * 3 * Kp * 2 + 255) & ~size_t(255);
  __nv_bfloat16* Bsl = reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(ws) + abytes);
  {
    SLU_REQUIRE(M <= 65535 && Kp / 64 <= 65535, "split grid too large");
    split_a_kernel<<<dim3((Kp / 4 + 255) / 256, M), 256, 0, st>>>(M, K, Kp, A, lda, Asl);
    check_launch("split_a_kernel");
    split_b_kernel<<<dim3((N + 63) / 64, Kp / 64), 256, 0, st>>>(K, N, Kp, B, ldb, Bsl);
    check_launch("split_b_kernel");
  }
  // 256-column tiles halve the operand traffic per flop; 128-column tiles
  // when the wider ones would leave most SMs idle
  const long long tiles256 = (long long)((N + 255) / 256) * ((M + BM - 1) / BM);
  if (tiles256 >= num_sms())
    launch_tc<256>(st, Asl, Bsl, M, N, Kp, alpha, beta, C, ldc, err);
  else
    launch_tc<128>(st, Asl, Bsl, M, N, Kp, alpha, beta, C, ldc, err);
}

}  // namespace slu
