// Block MVP that allocates nothing: scratch lives in a fixed device array.
//
// The regular entry point (bdda_op_mvp_device) grows the operator's MVP
// workspace with cudaMalloc on demand.  Some callers cannot let a library do
// that: host frameworks that own every byte of device memory through their
// own pool or arena, and latency-critical serving loops that must never enter
// the CUDA allocator (cudaMalloc/cudaFree can synchronise the device).  This
// variant runs the same five kernels with their two workspace buffers carved
// out of one file-scope __device__ array of kNoAllocScratchBytes.  A GPU
// reserves that array when this file's device code is loaded on it -- under
// CUDA's default lazy module loading, at the first call of the entry point
// there -- and keeps it until the process exits.  Only complex FP64 and FP32
// are offered (the double-float MVP is not).
//
// The array's host-side name is only a stand-in for the device symbol, so the
// device address is looked up once per device with cudaGetSymbolAddress, with
// that device current, the first time the entry point runs on it, and kept for
// the life of the process (a cudaDeviceReset after that is not supported).
// Make that first call at set-up, before any stream capture begins.  All calls share the one array
// and it keeps the last call's contents: calls whose work overlaps on the GPU
// (different streams, or different operators at the same time) race on it and
// must be ordered by the caller.  Nothing needs clearing between calls: every
// workspace element the kernels read was written earlier in the same call.
#include <mutex>
#include <string>

#include "../../include/bdda.h"
#include "op.hpp"

namespace bdda {
namespace {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Device address of the fixed scratch on the current device (looked up once).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return BDDA_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal outside the no-allocation scratch table");
    return BDDA_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (g_scratch_ptr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error(std::string("cudaGetSymbolAddress of the no-allocation scratch: ") + cudaGetErrorString(e));
      return BDDA_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return BDDA_OK;
}

template <typename T>
int mvp_noalloc(Op* op, const void* x, int ldx, void* y, int ldy, int L, const void* diag, const void* jpre,
                cudaStream_t st) {
  using C = typename cplx<T>::type;
  const int need = PrecInfo<T>::bit;
  if (!(op->prec & need)) {
    set_error("operator was created without the tables of this precision");
    return BDDA_ERR_INVALID;
  }
  const Occupancy& o = op->dip;
  if (L < 1 || ldx < op->f * o.nocc || ldy < op->f * o.nocc) {
    set_error("bad L or leading dimension");
    return BDDA_ERR_INVALID;
  }
  const MvpGeom g = op->geom<T>(o);
  const size_t b1 = align256(mvp_t1_elems(g, L) * sizeof(C));
  const size_t b2 = align256(mvp_t2_elems(g, L) * sizeof(C));
  if (b1 + b2 > kNoAllocScratchBytes) {
    set_error("no-allocation MVP needs " + std::to_string(b1 + b2) + " bytes of scratch for this box and nrhs; "
              "the fixed scratch holds " + std::to_string(kNoAllocScratchBytes) +
              " bytes (use bdda_op_mvp_device, or fewer right-hand sides per call)");
    return BDDA_ERR_INVALID;
  }
  void* base = nullptr;
  const int rc = scratch_address(&base);
  if (rc != BDDA_OK) return rc;
  C* t1 = static_cast<C*>(base);
  C* t2 = reinterpret_cast<C*>(static_cast<unsigned char*>(base) + b1);
  const cudaError_t e = launch_block_mvp<T>(g, op->tables<T>(), static_cast<const C*>(x), ldx, static_cast<C*>(y), ldy, L,
                                            static_cast<const C*>(diag), static_cast<const C*>(jpre), t1, t2, st,
                                            nullptr, nullptr);
  if (e != cudaSuccess) {
    set_error(std::string("no-allocation MVP launch: ") + cudaGetErrorString(e));
    return BDDA_ERR_CUDA;
  }
  return BDDA_OK;
}

}  // namespace
}  // namespace bdda

using namespace bdda;

extern "C" int bdda_op_mvp_device_noalloc(bdda_op* op, int prec, const void* x, int ldx, void* y, int ldy, int L,
                                          const void* diag, const void* jpre, void* stream) {
  if (!op || !x || !y) { set_error("null argument"); return BDDA_ERR_INVALID; }
  if (op->dip.nocc == 0) { set_error("no dipoles set on the operator"); return BDDA_ERR_INVALID; }
  std::lock_guard<std::mutex> lk(op->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : op->stream;
  if (prec == BDDA_PREC_FP64) return mvp_noalloc<double>(op, x, ldx, y, ldy, L, diag, jpre, st);
  if (prec == BDDA_PREC_FP32) return mvp_noalloc<float>(op, x, ldx, y, ldy, L, diag, jpre, st);
  set_error("prec must be BDDA_PREC_FP64 or BDDA_PREC_FP32");
  return BDDA_ERR_INVALID;
}
