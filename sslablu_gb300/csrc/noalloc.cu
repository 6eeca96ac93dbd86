// Allocation-free ULV solve: slu_ulv_solve_noalloc (include/slablu.h).
//
// Some callers cannot let a library allocate device memory on their solve
// path: a serving runtime that has reserved the GPU's memory for its own
// arena under a fixed budget, or a latency-critical loop where cudaMalloc's
// implicit synchronisation and unbounded latency are not acceptable.  For
// them this entry point runs the same float64 ULV solve as slu_ulv_solve but
// takes its scratch from a fixed array compiled into the library instead of
// the handle's grow-on-demand workspace.  It calls no cudaMalloc, cudaFree
// or allocating library routine.
//
// The scratch array is a file-scope __device__ variable, so every GPU that
// loads the library holds its kNoallocScratchBytes until the process exits.
// Host code cannot use the array's name as a device address (on the host it
// names a host-side stand-in); its device address is looked up once per
// device with cudaGetSymbolAddress on the first call made with that device
// current, and cached.
//
// All calls on a device share the one array: calls whose work overlaps on
// the GPU (different streams, or different host threads) race on it and must
// be serialised by the caller.  The array keeps the previous call's contents;
// the solve writes every scratch word before reading it, so nothing needs
// clearing between calls.
#include <mutex>

#include "abi_types.cuh"

namespace {

// 16 MiB: five N x nrhs float64 buffers, e.g. N = 4096 with up to 102
// right-hand sides, or N = 65536 with 6.
constexpr size_t kNoallocScratchBytes = size_t(16) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
// The kernels run on the handle's stream, so that stream must belong to the
// current device: the address of another device's copy of the array would be
// a peer address (a fault, or silent traffic over the interconnect).
void* noalloc_scratch_current_device(cudaStream_t st) {
  int dev = 0;
  SLU_CHECK_CUDA(cudaGetDevice(&dev));
  int sdev = dev;
  SLU_CHECK_CUDA(cudaStreamGetDevice(st, &sdev));
  SLU_REQUIRE(sdev == dev,
              "slu_ulv_solve_noalloc: the handle's stream belongs to device " +
                  std::to_string(sdev) + " but device " + std::to_string(dev) +
                  " is current; make the stream's device current first");
  SLU_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal out of range for the static scratch");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    SLU_CHECK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    SLU_REQUIRE(p != nullptr, "cudaGetSymbolAddress returned a null scratch address");
    g_scratch_addr[dev] = p;
  }
  return g_scratch_addr[dev];
}

}  // namespace

extern "C" {

int slu_ulv_solve_noalloc(slu_handle_t h, slu_hbs_t op, double* B, int ldb, int nrhs, int trans) {
  return slu::guard_call(h, [&] {
    SLU_REQUIRE(h && op && B, "null argument");
    SLU_REQUIRE(nrhs >= 1 && ldb >= nrhs, "bad right-hand side shape");
    const slu::Hbs& H = op->H;
    SLU_REQUIRE(H.has_ulv, "HBS operator has no ULV factorisation");
    const size_t need = slu::hbs_solve_scratch_bytes(H, nrhs, sizeof(double));
    if (need > kNoallocScratchBytes)
      throw slu::Error(SLU_ERR_ARG,
                       "slu_ulv_solve_noalloc: N x nrhs needs " + std::to_string(need) +
                           " scratch bytes, above the fixed limit of " +
                           std::to_string(kNoallocScratchBytes) +
                           " (use slu_ulv_solve, or fewer right-hand sides per call)");
    double* scratch = static_cast<double*>(noalloc_scratch_current_device(h->h.stream));
    slu::hbs_solve_scratch<double>(h->h.stream, H, trans != 0, B, ldb, nrhs, scratch);
  });
}

}  // extern "C"
