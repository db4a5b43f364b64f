// The operator object behind the C ABI (one lattice box + wavenumber).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "mvp.hpp"

namespace bdda {

// Thread-local last error text (bdda_last_error).
void set_error(const std::string& msg);
const char* last_error();

// RAII device buffer on the stream-ordered allocator: allocation and release
// are ordered on the owning stream (cudaMallocAsync / cudaFreeAsync), so
// freeing an operator never synchronises the device and concurrent solves on
// other streams keep running.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFreeAsync(p, stream);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t ensure(size_t b, cudaStream_t st) {
    if (b <= bytes) return cudaSuccess;
    release();
    stream = st;
    cudaError_t e = cudaMallocAsync(&p, b, st);
    if (e == cudaSuccess) bytes = b; else p = nullptr;
    return e;
  }
  template <typename X> X* as() const { return static_cast<X*>(p); }
};

// Signature of buffers' addresses and sizes, folded with the MurmurHash3
// 64-bit finaliser.  A graph captured with their pointers stays valid while
// it is unchanged: ensure() only reallocates to a larger size, so an equal
// (address, size) pair is the same live allocation.
inline unsigned long long sig_mix(unsigned long long h, unsigned long long v) {
  h ^= v;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdULL;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ULL;
  h ^= h >> 33;
  return h;
}
inline unsigned long long sig_add(unsigned long long h, const DevBuf& b) {
  return sig_mix(sig_mix(h, (unsigned long long)(uintptr_t)b.p), (unsigned long long)b.bytes);
}

// Keep freed stream-ordered memory in the device pool (no release to the OS
// at every synchronisation); called once per device.
void keep_pool_memory();

// Occupancy of the lattice by dipoles, on the device.
struct Occupancy {
  int nocc = 0;
  int ntiles = 0;             // (y, z-tile) pairs holding >= 1 dipole
  long long tile_rows = 0;    // their valid (y, z) columns
  DevBuf occ, tiles, tmask;
};

struct SolverWork;  // solver.cu

struct Op {
  int n[3] = {0, 0, 0};
  int P[3] = {0, 0, 0};
  int f = 3;
  double lf = 0, kr = 0, ki = 0;
  int prec = 0;  // bit mask BDDA_PREC_FP64 | BDDA_PREC_FP32
  // Axis plans per element width: [0] complex FP32 (the compile-time plan
  // tables' radix sequences, first-stage radices up to 32 along z), [1]
  // 16-byte FP64 / double-float (the 16-byte z table, radices <= 8 on the
  // single-line x / y axes).  Each set has its own Green spectrum order.
  AxisPlan plan[2][3];
  DevBuf tw64[3], tw32[3], twdf[3];
  DevBuf tw32p[3];  // complex FP32 twiddle pairs {wx, wx, wy, wy} of the packed z pass ([2] only)
  // staged twiddles (stage_twiddles) of the compile-time-plan kernels: complex
  // FP32 per axis, the packed z pass's pairs, the double-float z pass.  Every
  // DevBuf of the operator is released in ~Op, before its stream is destroyed.
  DevBuf tws32[3], tws32p, twsdf;
  DevBuf ghat64, ghat32, ghatdf;
  DevBuf kstat;     // int: status word of the pipelined z pass (take_kernel_status)
  Occupancy dip;    // dipole occupancy (set_dipoles)
  unsigned long long dip_epoch = 0;  // bumped whenever dip is rebuilt (captured MVPs hold its sizes)
  Occupancy cub;    // every cuboid site (the reference's MBT_fft_mvp vector)
  DevBuf t1[3], t2[3];   // MVP workspace per precision (0 = FP64, 1 = FP32, 2 = double-float)
  cudaStream_t stream = nullptr;
  KernelTimer timer;
  std::mutex mu;
  std::shared_ptr<SolverWork> solver;   // cached Krylov workspace (solver.cu)
  bool graphs = true;  // solvers' poll cycles as captured graphs (bdda_op_set_graphs)
  // Autotuned launch schedule of the complex FP32 block MVP, per nrhs
  // (bdda_op_set_autotune, bdda_op_get_tuning); candidate times in ms:
  // [0..7] pass B with 1 then 2 buffers x 2, 4, 8, 16 waves, [8..9] pass C
  // scalar / packed, [10..12] pass A at 5, 10, 20 CTAs per SM, [13] pass C
  // pipelined, [14..21] pass D as [0..7]; negative: not a candidate.
  struct TuneRec { MvpTune tune; float ms[22]; bool measured; };
  bool autotune = true;
  std::map<int, TuneRec> tuned;
  int zkern_force = -1;  // pass C kernel forced for every nrhs (bdda_op_set_z_kernel), -1: tuned / default
  int zstall = 0;        // test hook (bdda_op_test_z_stall)

  // signature of every buffer a block MVP's kernels are launched with
  unsigned long long buffer_sig() const {
    unsigned long long h = 0;
    for (int i = 0; i < 3; ++i) {
      for (const DevBuf* b : {&tw64[i], &tw32[i], &twdf[i], &tw32p[i], &tws32[i], &t1[i], &t2[i]}) h = sig_add(h, *b);
    }
    for (const DevBuf* b : {&ghat64, &ghat32, &ghatdf, &tws32p, &twsdf, &kstat, &dip.occ, &dip.tiles, &dip.tmask})
      h = sig_add(h, *b);
    return h;
  }

  MvpGeom geom(const Occupancy& o, int set) const {
    MvpGeom g;
    g.f = f;
    g.nx = n[0]; g.ny = n[1]; g.nz = n[2];
    g.nzp = (n[2] + 3) & ~3;  // 32-byte rows of complex FP32: aligned tile segments and column pairs
    g.Px = P[0]; g.Py = P[1]; g.Pz = P[2];
    g.px = plan[set][0]; g.py = plan[set][1]; g.pz = plan[set][2];
    g.nzt = (n[2] + kTZ - 1) / kTZ;
    g.gperm = 0;
    g.kstat = kstat.as<int>();
    g.zstall = zstall;
    g.ntiles = o.ntiles;
    g.tile_rows = o.tile_rows;
    g.occ = o.occ.as<int>();
    g.tiles = o.tiles.as<int>();
    g.tmask = o.tmask.as<unsigned char>();
    return g;
  }
  // complex FP32 tables: the Green spectrum is in the fused z pass's layout
  // (green_perm_radix); FP64 and double-float keep the natural one
  template <typename T> MvpGeom geom(const Occupancy& o) const {
    MvpGeom g = geom(o, sizeof(T) == sizeof(float) ? 0 : 1);
    g.gperm = sizeof(T) == sizeof(float) ? green_perm_radix(f, plan[0][2]) : 0;
    return g;
  }
  template <typename T> MvpPrec<T> tables() const;
  ~Op();
};

template <> inline MvpPrec<double> Op::tables<double>() const {
  return {tw64[0].as<double2>(), tw64[1].as<double2>(), tw64[2].as<double2>(), ghat64.as<double2>()};
}
template <> inline MvpPrec<float> Op::tables<float>() const {
  return {tw32[0].as<float2>(), tw32[1].as<float2>(), tw32[2].as<float2>(), ghat32.as<float2>(), tw32p[2].as<float4>(),
          tws32[0].as<float2>(), tws32[1].as<float2>(), tws32[2].as<float2>(), tws32p.as<float4>()};
}
template <> inline MvpPrec<dfl> Op::tables<dfl>() const {
  return {twdf[0].as<dfc>(), twdf[1].as<dfc>(), twdf[2].as<dfc>(), ghatdf.as<dfc>(), nullptr,
          nullptr, nullptr, twsdf.as<dfc>(), nullptr};
}

// Arithmetic of the block-MVP kernels for each table precision.
template <typename T> struct MvpArith { using type = T; };
template <> struct MvpArith<dfl> { using type = dfz; };

// Workspace slot and precision bit of each arithmetic type.
template <typename T> struct PrecInfo;
template <> struct PrecInfo<double> { static constexpr int slot = 0, bit = 1; };
template <> struct PrecInfo<float> { static constexpr int slot = 1, bit = 2; };
template <> struct PrecInfo<dfl> { static constexpr int slot = 2, bit = 4; };

// Make stream 'later' wait for the work enqueued so far on 'earlier'.
cudaError_t order_after(cudaStream_t later, cudaStream_t earlier);

// Wait for a stream without spinning a CPU core: records a blocking-sync event
// and sleeps on it, so many host threads can wait on concurrent solves.
cudaError_t wait_stream(cudaStream_t st);

// Build the occupancy tables from a host list of lattice addresses (null -> all sites).
int build_occupancy(Op* op, const int* address, int nocc, Occupancy* o);
// Reads and clears the operator's kernel status word (the pipelined z pass
// sets it when a bounded wait on a bulk copy gave up) once the work of stream
// st is done: BDDA_OK, or BDDA_ERR_CUDA with a message.
int take_kernel_status(Op* op, cudaStream_t st);

// y = [diag o x +] A_off x [o jpre] for L columns (device pointers, op->stream or st).
template <typename T>
int op_block_mvp(Op* op, const Occupancy& o, const typename cplx<T>::type* x, int ldx, typename cplx<T>::type* y, int ldy,
                 int L, const typename cplx<T>::type* diag, const typename cplx<T>::type* jpre, cudaStream_t st,
                 const int* done = nullptr);

}  // namespace bdda

// The opaque handle of the C ABI.
struct bdda_op : public bdda::Op {};
