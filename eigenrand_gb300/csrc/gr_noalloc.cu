// gr_raw_u64_noalloc: the raw-stream call for callers that cannot allocate
// device memory.
//
// Who needs it: code that must not call cudaMalloc on its sampling path —
// for example a host thread running under a real-time budget, or a plugin
// whose host framework owns all device memory and forbids the plugin from
// allocating behind its back.  Such a caller creates its engine once during
// set-up, passes its own output buffer on every call, and this entry point
// then allocates nothing: the jump-ahead scratch (lane prefixes, segment
// windows, jump polynomials) lives in one file-scope __device__ array that
// every GPU loading the library keeps until process exit.
//
// Limits: engines created with streams = 1 only, n <= GR_NOALLOC_MAX_DRAWS,
// at most kMaxSeg jump-ahead segments per call.  All calls share the array,
// so calls that overlap on the GPU (different streams, different threads)
// race on it and must be serialised by the caller.  The first call on a
// device performs the one-time set-up (looking up the array's device address
// and the kernel attributes); make that first call before any stream capture.
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
constexpr size_t kPrefixWords = (size_t)kLanes * kPrefixLen;              // 82368
constexpr size_t kSegWords = (size_t)(kMaxSeg - 1) * kLanes * kN;          // 38688
constexpr size_t kPolyWordsAll = (size_t)(kMaxSeg - 1) * kPolyWords;       // 9672
constexpr size_t kSnapWords = (sizeof(CallSnap) + 7) / 8 + 1;
constexpr size_t kScratchWords = kPrefixWords + kSegWords + kPolyWordsAll + kSnapWords;

}  // namespace

// ~1.0 MiB per device, held until process exit.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kScratchWords];

namespace {

struct DevScratch {
  uint64_t* base = nullptr;  // device address of g_noalloc_scratch on this device
  int64_t poly_J = -1;       // jump polynomials currently resident
  int poly_count = 0;
};

std::mutex g_mu;
std::map<int, DevScratch> g_dev;
std::map<int64_t, std::vector<Poly>> g_host_polys;  // host cache, by segment length

gr_status na_fail(gr_status s, const std::string& m) { return set_last_error(s, m); }

}  // namespace

extern "C" gr_status gr_raw_u64_noalloc(gr_engine* e, uint64_t* dev_out, size_t n, gr_stream_t stream) {
  if (!e || !dev_out) return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: NULL engine or output");
  if (gr_engine_streams(e) != 1)
    return na_fail(GR_ERR_UNSUPPORTED, "gr_raw_u64_noalloc: only engines created with streams = 1");
  if (n % kLanes) return na_fail(GR_ERR_INVALID, "gr_raw_u64_noalloc: n must be a multiple of 4");
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
    // one-time set-up for this device, with this device current
    void* p = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess)
      return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(err));
    ds.base = (uint64_t*)p;
  }
  uint64_t* prefix = ds.base;
  uint64_t* segwin = prefix + kPrefixWords;
  uint64_t* polys = segwin + kSegWords;
  CallSnap* snap = (CallSnap*)(polys + kPolyWordsAll);

  // segmentation: as the allocating path, but at most kMaxSeg segments
  const int64_t packets = (int64_t)(n / kLanes);
  int S = 1;
  int64_t J = packets;
  if (packets >= ((int64_t)1 << 17)) {
    int64_t j = (int64_t)1 << 14;
    while (j * 128 < packets) j <<= 1;
    while ((packets + j - 1) / j > kMaxSeg) j <<= 1;
    J = j;
    S = (int)((packets + j - 1) / j);
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
    if (ds.poly_J != J || ds.poly_count < S - 1) {
      auto& hp = g_host_polys[J];
      if ((int)hp.size() < kMaxSeg - 1) {
        if (charpoly_terms().size() != 284)
          return na_fail(GR_ERR_CUDA, "gr_raw_u64_noalloc: characteristic polynomial recovery failed");
        std::vector<uint64_t> exps(kMaxSeg - 1);
        for (int i = 0; i < kMaxSeg - 1; ++i) exps[i] = (uint64_t)(i + 1) * (uint64_t)J;
        pow_x_mod_many(exps, hp);
      }
      // pageable source: staged before cudaMemcpyAsync returns
      cudaError_t err = cudaMemcpyAsync(polys, hp.data(), sizeof(uint64_t) * kPolyWordsAll, cudaMemcpyHostToDevice, s);
      if (err != cudaSuccess)
        return na_fail(GR_ERR_CUDA, std::string("gr_raw_u64_noalloc: poly upload: ") + cudaGetErrorString(err));
      ds.poly_J = J;
      ds.poly_count = kMaxSeg - 1;
    }
    cudaError_t err = launch_prefix(p.eng, nullptr, 1, prefix, snap, s);
    if (err == cudaSuccess) err = launch_jump(prefix, polys, 1, S, segwin, s);
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
