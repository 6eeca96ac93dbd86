// Measured float64 FMA throughput of this GPU (slu_fp64_peak).
//
// The ULV solve's step kernels are bound by the float64 pipe at large
// right-hand-side counts, and the peaks measured for the roofline cover HBM
// bandwidth and bf16 tensor throughput only.  This kernel measures the
// float64 pipe the same way a copy measures HBM: every thread runs eight
// independent chains of dependent FMAs on register operands (no memory
// traffic inside the loop), the grid holds several CTAs per SM, and the time
// comes from CUDA events around the launch.  flops = 2 * FMAs.
#include "abi_types.cuh"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) fp64_fma_kernel(int iters, double a, double b,
                                                      double* __restrict__ sink) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  // a data-dependent store keeps the chains live; it never fires for the
  // contracting map used here (|x| stays below 1e30)
  if (s > 1e300) sink[blockIdx.x] = s;
}

}  // namespace

extern "C" {

int slu_fp64_peak(slu_handle_t h, int iters, double* tflops_out, double* ms_out) {
  return slu::guard_call(h, [&] {
    SLU_REQUIRE(h && tflops_out, "null argument");
    SLU_REQUIRE(iters >= 1 && iters <= (1 << 20), "iters out of range");
    cudaStream_t st = h->h.stream;
    const int ctas = 8 * slu::num_sms(), threads = 256;
    h->h.ws.reserve(sizeof(double) * ctas + 256, st);
    double* sink = h->h.ws.take<double>(ctas);
    cudaEvent_t e0, e1;
    SLU_CHECK_CUDA(cudaEventCreate(&e0));
    SLU_CHECK_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    for (int rep = 0; rep < 4; ++rep) {   // the first launch warms up; keep the best
      SLU_CHECK_CUDA(cudaEventRecord(e0, st));
      fp64_fma_kernel<<<ctas, threads, 0, st>>>(iters, 0.999999, 1e-7, sink);
      slu::check_launch("fp64_fma_kernel");
      SLU_CHECK_CUDA(cudaEventRecord(e1, st));
      SLU_CHECK_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      SLU_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * kChains * (double)iters * ctas * threads;
    *tflops_out = flops / (best * 1e-3) / 1e12;
    if (ms_out) *ms_out = best;
  });
}

}  // extern "C"
