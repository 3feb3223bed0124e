// gr_raw_u64_noalloc: the raw-stream call for callers that cannot allocate
// device memory.
//
// Who needs it: code that must not call cudaMalloc on its sampling path —
// for example a host thread running under a real-time budget, or a plugin
// whose host framework owns all device memory and forbids the plugin from
// allocating behind its back.  Such a caller creates its engine once during
// set-up, passes its own output buffer on every call, and this entry point
// then allocates nothing: the jump-ahead scratch (lane prefixes, segment
// windows) and every jump polynomial a call can need live in one file-scope
// __device__ array that every GPU loading the library keeps until process
// exit.
//
// Limits: engines created with streams = 1 only, n <= GR_NOALLOC_MAX_DRAWS,
// at most kMaxSeg jump-ahead segments per call (the allocating gr_raw_u64
// splits a long call into up to 128).  All calls share the array, so calls
// that overlap on the GPU (different streams, different threads) race on it
// and must be serialised by the caller.  The first call on a device performs
// the one-time set-up, with that device current: it looks up the array's
// device address, loads the kernels' code, computes the jump polynomials for
// every segment length a call can use and copies them into the array
// (synchronously).  Make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gpurand.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_poly.h"

using namespace gr;

namespace {

constexpr int kMaxSeg = 32;
// Segment lengths are powers of two: J = 2^kLogJMin .. 2^kLogJMax packets.
// The largest call (2^32 draws = 2^30 packets) in kMaxSeg segments needs
// J = 2^25.
constexpr int kLogJMin = 14;
constexpr int kLogJMax = 25;
constexpr int kJSets = kLogJMax - kLogJMin + 1;                             // 12
constexpr size_t kPrefixWords = (size_t)kLanes * kPrefixLen;              // 82368
constexpr size_t kSegWords = (size_t)(kMaxSeg - 1) * kLanes * kN;          // 38688
constexpr size_t kPolySetWords = (size_t)(kMaxSeg - 1) * kPolyWords;       // 9672 per J
constexpr size_t kPolyWordsAll = (size_t)kJSets * kPolySetWords;           // 116064
constexpr size_t kSnapWords = (sizeof(CallSnap) + 7) / 8 + 1;
constexpr size_t kScratchWords = kPrefixWords + kSegWords + kPolyWordsAll + kSnapWords;

}  // namespace

// ~1.9 MiB per device, held until process exit.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kScratchWords];

namespace {

struct DevScratch {
  uint64_t* base = nullptr;  // device address of g_noalloc_scratch on this device
};

std::mutex g_mu;
std::map<int, DevScratch> g_dev;
std::vector<Poly> g_host_polys;  // [kJSets][kMaxSeg - 1], computed once per process

gr_status na_fail(gr_status s, const std::string& m) { return set_last_error(s, m); }

// x^(i J) mod P(x) for every J = 2^kLogJMin .. 2^kLogJMax and i = 1 .. kMaxSeg - 1.
gr_status host_polys() {
  if (!g_host_polys.empty()) return GR_OK;
  if (charpoly_terms().size() != 284)
    return na_fail(GR_ERR_CUDA, "gr_raw_u64_noalloc: characteristic polynomial recovery failed");
  std::vector<uint64_t> exps;
  exps.reserve((size_t)kJSets * (kMaxSeg - 1));
  for (int lj = kLogJMin; lj <= kLogJMax; ++lj)
    for (int i = 1; i < kMaxSeg; ++i) exps.push_back((uint64_t)i << lj);
  pow_x_mod_many(exps, g_host_polys);
  return GR_OK;
}

// One-time set-up for the current device.
gr_status setup_device(DevScratch& ds) {
  void* p = nullptr;
  cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (err != cudaSuccess)
    return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(err));
  err = preload_raw_stream_kernels();
  if (err != cudaSuccess)
    return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: loading kernels: ") + cudaGetErrorString(err));
  gr_status st = host_polys();
  if (st != GR_OK) return st;
  uint64_t* polys = (uint64_t*)p + kPrefixWords + kSegWords;
  static_assert(sizeof(Poly) == kPolyWords * sizeof(uint64_t), "Poly is kPolyWords words");
  err = cudaMemcpy(polys, g_host_polys.data(), sizeof(uint64_t) * kPolyWordsAll, cudaMemcpyHostToDevice);
  if (err != cudaSuccess)
    return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: jump tables: ") + cudaGetErrorString(err));
  ds.base = (uint64_t*)p;
  return GR_OK;
}

}  // namespace

extern "C" gr_status gr_raw_u64_noalloc(gr_engine* e, uint64_t* dev_out, size_t n, gr_stream_t stream) {
  if (!e || !dev_out) return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: NULL engine or output");
  if (gr_engine_streams(e) != 1)
    return na_fail(GR_ERR_UNSUPPORTED, "gr_raw_u64_noalloc: only engines created with streams = 1");
  if (need_four_lanes(e, "gr_raw_u64_noalloc") != GR_OK) return GR_ERR_UNSUPPORTED;
  if (n % kLanes) return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: n must be a multiple of 4");
  if ((uintptr_t)dev_out % 16) return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: output must be 16-byte aligned");
  if (n > (size_t)GR_NOALLOC_MAX_DRAWS)
    return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: n exceeds GR_NOALLOC_MAX_DRAWS (2^32 draws); "
                                   "split the call");
  if (n == 0) return GR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return na_fail(GR_ERR_CUDA, "gr_raw_u64_noalloc: cudaGetDevice failed");

  std::lock_guard<std::mutex> lk(g_mu);
  DevScratch& ds = g_dev[dev];
  if (!ds.base) {
    gr_status st = setup_device(ds);
    if (st != GR_OK) return st;
  }
  uint64_t* prefix = ds.base;
  uint64_t* segwin = prefix + kPrefixWords;
  uint64_t* polys = segwin + kSegWords;
  CallSnap* snap = (CallSnap*)(polys + kPolyWordsAll);

  // segmentation: as the allocating path, but at most kMaxSeg segments
  const int64_t packets = (int64_t)(n / kLanes);
  int S = 1;
  int64_t J = packets;
  int lj = 0;
  if (packets >= ((int64_t)1 << 17)) {
    lj = kLogJMin;
    while (((int64_t)128 << lj) < packets) ++lj;
    while ((packets + ((int64_t)1 << lj) - 1) >> lj > kMaxSeg) ++lj;
    if (lj > kLogJMax) return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: call too long for the jump tables");
    J = (int64_t)1 << lj;
    S = (int)((packets + J - 1) / J);
  }
  Plan p{};
  p.eng = engine_state_ptr(e);
  p.gen = nullptr;
  p.K = 1;
  p.S = S;
  p.J = J;
  p.gran = 4;
  p.gran_per_k = packets;
  p.gran_rem = 0;
  p.out = dev_out;
  if (S > 1) {
    // the tables for this J: x^(i J) mod P for i = 1 .. kMaxSeg - 1
    const uint64_t* pj = polys + (size_t)(lj - kLogJMin) * kPolySetWords;
    cudaError_t err = launch_prefix(p.eng, nullptr, 1, prefix, snap, s);
    if (err == cudaSuccess) err = launch_jump(prefix, pj, 1, S, segwin, s);
    if (err != cudaSuccess)
      return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: jump-ahead: ") + cudaGetErrorString(err));
    p.segwin = segwin;
    p.prefix = prefix;
  }
  DistParams dp{};
  dp.kind = kRawKind;
  dp.dtype = GR_U64;
  cudaError_t err = launch_direct(p, dp, snap, s);
  if (err != cudaSuccess)
    return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: sampling kernel: ") + cudaGetErrorString(err));
  return GR_OK;
}
