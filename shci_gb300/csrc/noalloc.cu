// shci_hamiltonian_elems_noalloc: matrix elements for callers that cannot allocate device
// memory.
//
// Some host programs cannot call cudaMalloc while they run this library: a process whose
// device memory is already fully reserved by another framework's caching allocator (every
// new cudaMalloc would fail or force that allocator to release memory), code that runs under
// a fixed memory budget enforced outside CUDA, or an embedding that forbids device
// allocation after start-up.  shci_hamiltonian_elems stages its inputs and results in
// device buffers it allocates per call.  This variant stages them in one file-scope device
// array of fixed size instead, so a call allocates nothing.
//
// Limits and sharing rules:
//   - at most kMaxPairs (65,536) det pairs per call; larger requests are rejected with
//     SHCI_ERR_ARG (split them into several calls);
//   - the array is part of every GPU that loads this library and stays resident until the
//     process exits (2.5 MiB: 4 x 8 bytes of det strings + 8 bytes of result per pair);
//   - all calls in the process share the one array per device: two calls whose work overlaps
//     on the GPU (for example from two host threads or two contexts on one device) race and
//     corrupt each other's results; serialise them;
//   - every call overwrites the slots it uses before reading them, so nothing in the array
//     has to start at zero, and a call never sees results of an earlier call;
//   - every call looks up the array's device address in the calling thread's current
//     context (cudaGetSymbolAddress, no allocation), so a device reset or a different
//     context on the same device never sees a stale address; the first call on a device can
//     load the library's device code, so make it before any stream capture.
#include <cstring>

#include "ctx.h"
#include "kernels.h"

namespace shci {

namespace {

constexpr size_t kMaxPairs = 65536;
constexpr size_t kScratchBytes = kMaxPairs * (4 * sizeof(uint64_t) + sizeof(double));
constexpr int kMaxDevices = 64;

// Device scratch: [4 * kMaxPairs] u64 det strings (up_i, dn_i, up_j, dn_j), then
// [kMaxPairs] doubles of results.  In host code this name is only a stand-in for the symbol;
// its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_elem_scratch[kScratchBytes];

// Device address of g_elem_scratch in the current context (the caller has made `device`
// current).  Looked up on every call: a cached address would outlive a cudaDeviceReset or
// belong to another context of the same device.
void* scratch_address(int device) {
  if (device < 0 || device >= kMaxDevices) throw ArgError("device ordinal out of range");
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_elem_scratch);
  if (e != cudaSuccess) throw CudaError(e, "cudaGetSymbolAddress(g_elem_scratch)");
  return p;
}

__global__ void k_elems_scratch(DevIntegrals I, unsigned char* scratch, size_t n) {
  const uint64_t* ui = reinterpret_cast<const uint64_t*>(scratch);
  const uint64_t* di = ui + kMaxPairs;
  const uint64_t* uj = ui + 2 * kMaxPairs;
  const uint64_t* dj = ui + 3 * kMaxPairs;
  double* out = reinterpret_cast<double*>(scratch + 4 * kMaxPairs * sizeof(uint64_t));
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    if (ui[k] == uj[k] && di[k] == dj[k]) out[k] = h_diag(I, ui[k], di[k]);
    else out[k] = h_offdiag(I, ui[k], di[k], uj[k], dj[k]);
  }
}

}  // namespace

void hamiltonian_elems_noalloc(shci_ctx* c, const uint64_t* ui, const uint64_t* di,
                               const uint64_t* uj, const uint64_t* dj, size_t n, double* out) {
  if (n > kMaxPairs)
    throw ArgError("shci_hamiltonian_elems_noalloc takes at most 65536 det pairs per call (got " +
                   std::to_string(n) + "); split the request");
  if (n == 0) return;
  if (!ui || !di || !uj || !dj || !out) throw ArgError("null input or output pointer");
  unsigned char* base = static_cast<unsigned char*>(scratch_address(c->device));
  uint64_t* s = reinterpret_cast<uint64_t*>(base);
  cudaStream_t st = c->stream;
  SHCI_CUDA(cudaMemcpyAsync(s, ui, n * 8, cudaMemcpyHostToDevice, st));
  SHCI_CUDA(cudaMemcpyAsync(s + kMaxPairs, di, n * 8, cudaMemcpyHostToDevice, st));
  SHCI_CUDA(cudaMemcpyAsync(s + 2 * kMaxPairs, uj, n * 8, cudaMemcpyHostToDevice, st));
  SHCI_CUDA(cudaMemcpyAsync(s + 3 * kMaxPairs, dj, n * 8, cudaMemcpyHostToDevice, st));
  k_elems_scratch<<<grid_for(n, 128), 128, 0, st>>>(c->dI, base, n);
  SHCI_LAUNCH_CHECK();
  SHCI_CUDA(cudaMemcpyAsync(out, base + 4 * kMaxPairs * sizeof(uint64_t), n * 8,
                            cudaMemcpyDeviceToHost, st));
  SHCI_CUDA(cudaStreamSynchronize(st));
  c->launches += 1;
}

}  // namespace shci
