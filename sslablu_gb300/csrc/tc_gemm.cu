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
// one tcgen05 GEMM over the concatenated K: float32 inside 512-term chunks,
// double-float (float32 pairs, error-free TwoSum) across chunks.  Relative accuracy is that of a float32 GEMM of depth
// 512, which is what the refinement-driven mixed path needs; the float64 path
// never uses this kernel.
//
// Kernel: one CTA per 128 x 128 output tile, 192 threads.
//   warp 4 lane 0 : TMA producer, 3-stage ring of (A, B) 128 x 64 bf16 slabs
//                   (128B-swizzled, one mbarrier per stage, complete_tx)
//   warp 5 lane 0 : MMA issuer, tcgen05.mma.cta_group::1.kind::f16
//                   (M=128, N=128, K=16 per instruction); K runs in chunks of
//                   512 into two ping-pong float32 TMEM accumulators, and
//                   tcgen05.commit frees each stage / publishes each chunk;
//                   warp 5 also allocates and frees the 256 TMEM columns
//   warps 0-3     : epilogue, tcgen05.ld 32x32b rows of each finished chunk
//                   added (error-free TwoSum, float32 ops) into a
//                   double-float tile in shared memory, then C in float64
// Every mbarrier wait is bounded; on timeout the kernel records an error word,
// drains what it issued (again bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <mutex>

#include "slablu_internal.cuh"

namespace slu {
namespace {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3;
constexpr int TILE_BYTES = BM * BK * 2;          // 16 KB per operand slab
constexpr int STAGE_BYTES = 2 * TILE_BYTES;      // A + B
constexpr int ACC_BYTES = BM * BN * 8;           // (hi, lo) float pair tile accumulator
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + ACC_BYTES + 1024;
constexpr uint32_t TMEM_COLS = 2 * BN;           // two float32 accumulators (ping-pong)
constexpr int CHUNK = 8;                         // k-tiles (of BK) per float32 chunk
constexpr int kThreadsTC = 192;                  // warps 0-3 epilogue, 4 TMA, 5 MMA
constexpr long long kWaitLimit = 1LL << 22;      // try_wait rounds before giving up

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

// Instruction descriptor, kind::f16: D f32, A/B bf16, both K-major, M = 128, N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
}

// K is consumed in chunks of CHUNK k-tiles.  Chunk c accumulates in float32
// TMEM accumulator c % 2; the epilogue warps add each finished chunk into a
// double-float tile in shared memory while the MMA warp fills the other
// accumulator, so float32 rounding acts only within 512-term chunks.  (The
// drain uses float32 arithmetic: GB300's float64 pipe is ~1/64 of it.)
__global__ void __launch_bounds__(kThreadsTC, 1)
tc_gemm_bf16_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    int M, int N, int Kp, double alpha, double beta, double* __restrict__ C,
                    int ldc, unsigned int* __restrict__ err) {
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
  // double-float accumulator, [BN][BM] column-major so a warp's 32 rows are
  // consecutive: hi at acc_hi, lo at acc_lo
  float* acc_hi = reinterpret_cast<float*>(smem + STAGES * STAGE_BYTES);
  float* acc_lo = acc_hi + BM * BN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int KT = Kp / BK;
  const int NC = (KT + CHUNK - 1) / CHUNK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&ready_bar[a], 1);
      mbar_init(&drained_bar[a], 128);
    }
    s_fail = 0;
    s_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  if (warp == 4) {
    // ---------------- TMA producer
    if (lane == 0) {
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % STAGES;
        if (kt >= STAGES && !mbar_wait(&empty_bar[s], ((kt / STAGES) + 1) & 1)) {
          s_fail = 1;
          break;
        }
        unsigned char* a = smem + s * STAGE_BYTES;
        unsigned char* b = a + TILE_BYTES;
        mbar_expect_tx(&full_bar[s], STAGE_BYTES);
        tma_load_2d(a, &tmA, kt * BK, m0, &full_bar[s]);
        tma_load_2d(b, &tmB, kt * BK, n0, &full_bar[s]);
        s_issued = kt + 1;
      }
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer
    if (lane == 0) {
      int kt = 0;
      bool fail = false;
      for (int c = 0; c < NC && !fail; ++c) {
        const int a = c & 1;
        if (c >= 2 && !mbar_wait(&drained_bar[a], ((c >> 1) - 1) & 1)) {
          fail = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dacc = tmem + (uint32_t)(a * BN);
        for (int j = 0; j < CHUNK && kt < KT; ++j, ++kt) {
          const int s = kt % STAGES;
          if (!mbar_wait(&full_bar[s], (kt / STAGES) & 1)) {
            fail = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
          const uint32_t sb = sa + TILE_BYTES;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16(dacc, smem_desc(sa + kk * 32), smem_desc(sb + kk * 32), (j | kk) != 0);
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
    // ---------------- epilogue warps 0-3: TMEM lanes 32*warp .. 32*warp+31
    const int r = warp * 32 + lane;  // tile row owned by this thread
    for (int cidx = 0; cidx < BN; ++cidx) acc_hi[cidx * BM + r] = acc_lo[cidx * BM + r] = 0.0f;
    bool fail = false;
    for (int c = 0; c < NC; ++c) {
      const int a = c & 1;
      if (!mbar_wait(&ready_bar[a], (c >> 1) & 1)) {
        fail = true;
        break;
      }
      if (s_fail) {
        fail = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t v[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(a * BN + c0), v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          // error-free TwoSum of (hi, v); the rounding error goes to lo
          const int idx = (c0 + j) * BM + r;
          const float x = __uint_as_float(v[j]);
          const float h = acc_hi[idx];
          const float sum = h + x;
          const float bb = sum - h;
          const float e = (h - (sum - bb)) + (x - bb);
          acc_hi[idx] = sum;
          acc_lo[idx] += e;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&drained_bar[a]);
    }
    if (fail) {
      if (lane == 0 && err) atomicOr(err, 1u);
    } else {
      const int row = m0 + r;
      if (row < M) {
        double* crow = C + (long long)row * ldc;
        for (int cidx = 0; cidx < BN; ++cidx) {
          const int col = n0 + cidx;
          if (col < N) {
            const double v =
                alpha * ((double)acc_hi[cidx * BM + r] + (double)acc_lo[cidx * BM + r]);
            crow[col] = (beta == 0.0) ? v : fma(beta, crow[col], v);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 5)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
}

// ---------------------------------------------------------------- splitting
// Slices of x: s0 = bf16(x), s1 = bf16(x - s0), s2 = bf16(x - s0 - s1).
__device__ __forceinline__ void split3(double x, __nv_bfloat16& s0, __nv_bfloat16& s1,
                                       __nv_bfloat16& s2) {
  s0 = __double2bfloat16(x);
  double r = x - (double)__bfloat162float(s0);
  s1 = __double2bfloat16(r);
  r -= (double)__bfloat162float(s1);
  s2 = __double2bfloat16(r);
}

// Slice order of the six cross products along the concatenated K.
__constant__ int kTermA[6] = {0, 0, 1, 0, 1, 2};
__constant__ int kTermB[6] = {0, 1, 0, 2, 1, 0};

// A (M x K row-major, float64) -> Acat (M x 6*Kp bf16): block t holds slice kTermA[t].
__global__ void split_a_kernel(int M, int K, int Kp, const double* __restrict__ A, int lda,
                               __nv_bfloat16* __restrict__ out) {
  const long long total = (long long)M * Kp;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / Kp), k = (int)(e % Kp);
    __nv_bfloat16 s[3];
    if (k < K) split3(A[(long long)i * lda + k], s[0], s[1], s[2]);
    else s[0] = s[1] = s[2] = __double2bfloat16(0.0);
    __nv_bfloat16* row = out + (long long)i * 6 * Kp;
#pragma unroll
    for (int t = 0; t < 6; ++t) row[t * Kp + k] = s[kTermA[t]];
  }
}

// B (K x N row-major, float64) -> Bcat (N x 6*Kp bf16, K-major): block t holds slice kTermB[t].
__global__ void split_b_kernel(int K, int N, int Kp, const double* __restrict__ B, int ldb,
                               __nv_bfloat16* __restrict__ out) {
  __shared__ double tile[32][33];
  const int k0 = blockIdx.y * 32, n0 = blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int k = k0 + r, n = n0 + threadIdx.x;
    tile[r][threadIdx.x] = (k < K && n < N) ? B[(long long)k * ldb + n] : 0.0;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int n = n0 + r, k = k0 + threadIdx.x;
    if (n >= N || k >= Kp) continue;
    __nv_bfloat16 s[3];
    split3(tile[threadIdx.x][r], s[0], s[1], s[2]);
    __nv_bfloat16* row = out + (long long)n * 6 * Kp;
#pragma unroll
    for (int t = 0; t < 6; ++t) row[t * Kp + k] = s[kTermB[t]];
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

// rows x cols bf16 matrix, row pitch cols (K-major), box 64 x 128, 128B swizzle.
CUtensorMap make_map(const void* base, int rows, long long cols) {
  SLU_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0, "TMA base must be 16-byte aligned");
  SLU_REQUIRE((cols * 2) % 16 == 0, "TMA row pitch must be a multiple of 16 bytes");
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {BK, 128};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(SLU_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return m;
}

}  // namespace

size_t tc_gemm_workspace_bytes(int M, int N, int K) {
  const long long Kp = ((long long)K + BK - 1) / BK * BK;
  return (size_t)(6 * Kp * 2) * ((size_t)M + N) + 2 * 256;
}

// C = alpha A B + beta C with split-BF16x3 tcgen05 products (float32 accumulation).
// ws: tc_gemm_workspace_bytes(M, N, K) bytes; err: device word set on a wait timeout.
void tc_gemm_split3(cudaStream_t st, int M, int N, int K, double alpha, const double* A, int lda,
                    const double* B, int ldb, double beta, double* C, int ldc, void* ws,
                    unsigned int* err) {
  if (M <= 0 || N <= 0) return;
  SLU_REQUIRE(K >= 1, "K must be positive");
  const int Kp = (K + BK - 1) / BK * BK;
  const long long Kc = 6LL * Kp;
  SLU_REQUIRE(Kc < (1LL << 31), "K too large");
  __nv_bfloat16* Acat = reinterpret_cast<__nv_bfloat16*>(ws);
  size_t abytes = ((size_t)M * Kc * 2 + 255) & ~size_t(255);
  __nv_bfloat16* Bcat = reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(ws) + abytes);
  {
    long long total = (long long)M * Kp;
    int g = (int)std::min<long long>((total + 255) / 256, 8LL * num_sms());
    split_a_kernel<<<g, 256, 0, st>>>(M, K, Kp, A, lda, Acat);
    check_launch("split_a_kernel");
    dim3 gb((N + 31) / 32, (Kp + 31) / 32);
    split_b_kernel<<<gb, dim3(32, 8), 0, st>>>(K, N, Kp, B, ldb, Bcat);
    check_launch("split_b_kernel");
  }
  CUtensorMap ma = make_map(Acat, M, Kc);
  CUtensorMap mb = make_map(Bcat, N, Kc);
  static bool attr = false;
  if (!attr) {
    SLU_CHECK_CUDA(cudaFuncSetAttribute(tc_gemm_bf16_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    attr = true;
  }
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
  tc_gemm_bf16_kernel<<<grid, kThreadsTC, SMEM_BYTES, st>>>(ma, mb, M, N, (int)Kc, alpha, beta, C,
                                                            ldc, err);
  check_launch("tc_gemm_bf16_kernel");
}

}  // namespace slu
