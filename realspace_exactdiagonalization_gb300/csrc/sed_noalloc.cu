// sed_noalloc.cu -- H|psi> without any device allocation.
//
// Some callers cannot call cudaMalloc when they apply the Hamiltonian:
//   * a host that hands all device memory to its own pool (a Julia process
//     using CUDA.jl's pool, or PyTorch's caching allocator) and may not grab
//     memory behind that allocator's back;
//   * a latency-critical loop (a serving loop, a solver inside another
//     program's time step) where cudaMalloc's implicit device-wide
//     synchronisation would stall unrelated streams;
//   * code that must not allocate once set-up is over (fixed memory budget).
// sed_op_apply allocates its two orbit-indexed work vectors on first use.
// This variant takes them from a fixed array in device global memory instead,
// declared below at file scope, so the call itself allocates nothing.
//
// Limits and rules of use:
//   * the scratch holds two complex128 vectors of up to kNoAllocMaxOrbits
//     (1,048,576) orbits: 32 MiB that every GPU loading this library keeps
//     until the process exits; larger sectors are rejected (SED_ERR_LIMIT);
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (which may load the module); make that first call
//     before any stream capture;
//   * the call never runs the gather's launch-shape autotuner (whose timing
//     runs wait on the host): it uses the operator's shape if one is chosen
//     or pinned, else the shape remembered for the same catalog shape, else
//     the default of one thread per row and 512 threads per block;
//   * every call shares the one array: calls that overlap on the GPU (two
//     streams, two threads, two operators) race and must be serialised by the
//     caller.  Each call clears what it needs to start at zero, so a call
//     never sees the previous call's contents.
#include <mutex>

#include "../../include/sed_capi.h"
#include "sed_handles.cuh"
#include "sed_internal.cuh"

namespace sed {

void expand_vec(const SectorImpl& S, const double* xsec, double* xpad, cudaStream_t s);
void compress_vec(const SectorImpl& S, const double* ypad, double* ysec, cudaStream_t s);

static constexpr int64_t kNoAllocMaxOrbits = int64_t(1) << 20;

// [0, kNoAllocMaxOrbits): the scaled input; [kNoAllocMaxOrbits, 2x): the
// expanded input, then the orbit-indexed output.
static __device__ __align__(256) double2 g_noalloc_scratch[2 * kNoAllocMaxOrbits];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[256] = {};

// Device address of the scratch on the current device (host code cannot use
// the symbol itself: on the host it names a stand-in, not device memory).
static double2* noalloc_scratch_current_device() {
  int dev = 0;
  SED_CUDA(cudaGetDevice(&dev));
  SED_REQUIRE(dev >= 0 && dev < 256, SED_ERR_LIMIT, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      throw Error{SED_ERR_CUDA, std::string("cudaGetSymbolAddress of the no-alloc scratch failed: ") +
                                    cudaGetErrorString(e)};
    g_noalloc_addr[dev] = p;
  }
  return static_cast<double2*>(g_noalloc_addr[dev]);
}

void op_apply_noalloc(OpImpl& op, const double* x, double* y, int64_t n) {
  const SectorImpl& S = *op.sec;
  SED_REQUIRE(x != nullptr && y != nullptr, SED_ERR_ARG, "x and y must not be NULL");
  SED_REQUIRE(n == S.dim, SED_ERR_ARG, "vector length must equal the sector dimension");
  const int64_t n_orb = S.cat->n_orbits;
  SED_REQUIRE(n_orb <= kNoAllocMaxOrbits, SED_ERR_LIMIT,
              "sed_op_apply_noalloc: the catalog has " + std::to_string(n_orb) +
                  " orbits, above the fixed scratch limit of 1048576 orbits; use sed_op_apply");
  double2* scratch = noalloc_scratch_current_device();
  double* xs = reinterpret_cast<double*>(scratch);
  double* pad = reinterpret_cast<double*>(scratch + kNoAllocMaxOrbits);
  cudaStream_t s = op.stream;
  expand_vec(S, x, pad, s);  // zeroes the n_orb entries, then scatters x
  op_scale_to_xs(op, pad, xs, s);
  op_apply_orbit_untuned(op, xs, pad, s);
  compress_vec(S, pad, y, s);
}

}  // namespace sed

extern "C" int sed_op_apply_noalloc(sed_op* op, const double* x_dev, double* y_dev, int64_t n) {
  try {
    SED_REQUIRE(op != nullptr, SED_ERR_ARG, "NULL operator");
    sed::op_apply_noalloc(*op->p, x_dev, y_dev, n);
    return SED_OK;
  } catch (const sed::Error& e) {
    sed::set_error(e.msg);
    return e.code;
  } catch (const std::exception& e) {
    sed::set_error(e.what());
    return SED_ERR_ARG;
  }
}
