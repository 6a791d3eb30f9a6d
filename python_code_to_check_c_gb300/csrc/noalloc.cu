// tdcc_dipole_noalloc: the dipole expectation value of tdcc_dipole computed
// without allocating device memory.
//
// Who needs it: callers that may not call cudaMalloc -- code running while a
// CUDA graph is being captured by someone else, plugins handed a fixed memory
// budget by a host framework that owns every allocation, or a process that
// must not grow its footprint after start-up.  They pass their own inputs and
// output; the intermediates (density blocks Dij, Dab, Dai and three small
// products) live in the static device array below instead of a workspace.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tdcc.h"
#include "engine.h"

namespace tdcc {
void build_density(Program& p, int n_mu);
}

using namespace tdcc;

namespace {

// Size limits of the no-allocation path.
constexpr int kNoAllocMaxO = 64;
constexpr int kNoAllocMaxV = 256;
// Dij (o*o) + Dab (v*v) + Dai (v*o) + three products (v*v, v*v, o*o), complex128:
// 221,184 elements = 3.375 MiB, held on every device that loads this module.
constexpr size_t kScratchElems = 2ull * kNoAllocMaxO * kNoAllocMaxO +
                                 3ull * kNoAllocMaxV * kNoAllocMaxV +
                                 (size_t)kNoAllocMaxO * kNoAllocMaxV;

__device__ __align__(256) double2 g_dipole_scratch[kScratchElems];

// Device addresses of g_dipole_scratch, one per device (host code cannot use
// the symbol itself: on the host it is only a stand-in for the device array).
// Looked up once per device and kept for the life of the process; a device
// reset (cudaDeviceReset) reloads the module, after which a kept address
// would be stale, so resetting a device between calls is not supported.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double2* g_scratch_addr[kMaxDevices] = {};

int fail_na(int code, const std::string& m) {
  set_error(m);
  return code;
}

}  // namespace

extern "C" int tdcc_dipole_noalloc(int o, int v, const void* t1, const void* t2, const void* l1,
                                   const void* l2, const double* mu, int n_mu, void* mu_out,
                                   void* stream) {
  if (o < 1 || v < 1) return fail_na(TDCC_ERR_ARG, "o and v must be >= 1");
  if (o > kNoAllocMaxO || v > kNoAllocMaxV)
    return fail_na(TDCC_ERR_LIMIT, "tdcc_dipole_noalloc supports o <= " + std::to_string(kNoAllocMaxO) +
                                       " and v <= " + std::to_string(kNoAllocMaxV) + " (got o=" +
                                       std::to_string(o) + ", v=" + std::to_string(v) +
                                       "); use tdcc_dipole for larger systems");
  if (n_mu < 1 || n_mu > 3) return fail_na(TDCC_ERR_ARG, "n_mu must be 1..3");
  if (!t1 || !t2 || !l1 || !l2 || !mu || !mu_out) return fail_na(TDCC_ERR_ARG, "NULL argument");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail_na(TDCC_ERR_CUDA, "cudaGetDevice failed or device index out of range");
  }
  double2* scratch = nullptr;
  {
    // one-time set-up per device, with that device current
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_dipole_scratch);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return fail_na(TDCC_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      }
      g_scratch_addr[dev] = static_cast<double2*>(p);
    }
    scratch = g_scratch_addr[dev];
  }

  try {
    Program p(Dims{o, v, o + v}, "density_noalloc");
    build_density(p, n_mu);
    std::vector<void*> bases(p.slots.size(), nullptr);
    size_t off = 0;
    for (size_t i = kNumFixedSlots; i < p.slots.size(); ++i) {
      if (p.slots[i].dt != C64) return fail_na(TDCC_ERR_STATE, "unexpected real workspace in density program");
      bases[i] = scratch + off;
      off += (size_t)p.slots[i].numel;
    }
    if (off > kScratchElems) return fail_na(TDCC_ERR_LIMIT, "density scratch exceeds the static array");
    bases[S_T1] = const_cast<void*>(t1);
    bases[S_T2] = const_cast<void*>(t2);
    bases[S_L1] = const_cast<void*>(l1);
    bases[S_L2] = const_cast<void*>(l2);
    bases[S_MU] = const_cast<double*>(mu);
    bases[S_RES] = mu_out;
    // Every scratch block is overwritten (or zero-filled for split-K sums)
    // by its first op, so stale contents of an earlier call do not matter.
    if (p.run(bases, static_cast<cudaStream_t>(stream), Program::ALL) != cudaSuccess) return TDCC_ERR_CUDA;
  } catch (const std::exception& ex) {
    return fail_na(TDCC_ERR_CUDA, ex.what());
  }
  return TDCC_OK;
}
