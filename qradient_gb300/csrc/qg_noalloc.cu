// qg_grad_noalloc: McClean / QAOA adjoint gradient with library-owned scratch.
//
// Some callers cannot call cudaMalloc on the path where they need a
// gradient: plug-ins whose host process owns every device allocation
// through its own pool (it reserves the device memory up front, so a
// library allocation either fails or escapes the host's accounting), and
// real-time loops that forbid allocation after start-up (cudaMalloc may
// synchronise the device and takes an unbounded time).  This entry point
// takes the same inputs and outputs as qg_grad but needs no workspace from
// the caller: its scratch is one file-scope device array, which every GPU
// that loads the library's device code holds until the process exits.
// With CUDA's lazy module loading that happens at the library's first
// kernel launch or symbol lookup on the device, not when the shared
// library is opened.
//
// The array is QG_NOALLOC_SCRATCH_BYTES (16 MiB).  A circuit fits when its
// uncompute-mode workspace (qg_workspace_size with QG_OP_GRAD_UNCOMPUTE)
// does; larger circuits get QG_ERR_UNSUPPORTED before anything is launched.
// Nothing in the scratch has to start at zero: the gradient pass clears its
// partial sums itself and writes every state before reading it.  All calls
// on a device share the array and it keeps the previous call's contents, so
// calls whose work overlaps on the GPU (different streams, or several host
// threads) race; callers must order them, for example on one stream.
//
// The array's device address is looked up once per device (the first call
// on that device, with it current) and cached for the life of the process.
// A context reset (cudaDeviceReset, or a primary context that is released
// and created again) reloads the module, possibly at another address, and
// invalidates the cached one: such a caller must not use this entry point
// after the reset.
#include <cuda_runtime.h>

#include <mutex>

#include <stdio.h>

#include "../../include/qgrad.h"
#include "qg_kernels.h"

namespace {

constexpr size_t kScratchBytes = QG_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// Device scratch.  In host code this symbol is only a handle for
// cudaGetSymbolAddress, never an address a kernel may use.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device with that device current.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return QG_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return QG_ERR_CUDA;
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return QG_OK;
}

}  // namespace

extern "C" int qg_grad_noalloc(const qg_circuit* c, int dtype, const double* params_dev, const void* ini_state_dev,
                               double* expec_dev, double* grad_dev, qg_stream stream) {
  size_t need = 0;
  int st = qg_workspace_size(c, dtype, QG_OP_GRAD_UNCOMPUTE, &need);
  if (st != QG_OK) return st;
  if (need > kScratchBytes) {
    char msg[256];
    snprintf(msg, sizeof msg,
             "qg_grad_noalloc: this circuit needs %zu bytes of scratch, above the fixed %zu-byte array; "
             "use qg_grad with a caller workspace",
             need, kScratchBytes);
    return qg::set_last_error(QG_ERR_UNSUPPORTED, msg);
  }
  void* scratch = nullptr;
  st = scratch_address(&scratch);
  if (st != QG_OK) return qg::set_last_error(st, "qg_grad_noalloc: cudaGetSymbolAddress of the scratch array failed");
  return qg_grad(c, dtype, QG_OP_GRAD_UNCOMPUTE, params_dev, ini_state_dev, scratch, kScratchBytes, expec_dev,
                 grad_dev, stream);
}
