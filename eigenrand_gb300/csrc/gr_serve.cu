// Serving loop over per-client device-resident engines (include/gpurand.h).
//
// Host-side scheduler only: requests are admitted by gr::Admission (arrival
// order, one request per client at a time, device-memory budget, stream
// slots), launched on a free slot's stream through the library's own C ABI,
// and harvested by polling one event per slot.  Outputs come from a
// stream-ordered memory pool reserved for the server.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gpurand.h"
#include "gr_admit.h"
#include "gr_internal.h"
#include "gr_kernels.cuh"
#include "gr_mv.cuh"

using namespace gr;

namespace {

gr_status sfail(gr_status s, const std::string& m) { return set_last_error(s, m); }

#define SV_CUDA(call)                                                                                  \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) return set_last_error(GR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2 };

struct ServeReq {
  gr_request r;
  uint64_t ticket = 0;
  uint64_t gen = 0;   // scalars generated (count rounded up)
  uint64_t units = 0; // value passed to the sampling call (samples for MvNormal)
  size_t bytes = 0;
  size_t charged = 0;  // bytes held in the admission budget (from admission to release)
  void* dev_out = nullptr;
  int slot = -1;
  int state = kQueued;
  bool cancelled = false;  // running when cancelled: freed and reported as such on completion
  bool reported = false;
  gr_status status = GR_OK;
  double admitted = 0, completed = 0;
};

size_t elem_bytes(int dtype) { return dtype == GR_F64 ? 8 : 4; }

bool serve_kind_ok(int kind) {
  return (kind >= GR_UNIFORM_REAL && kind <= GR_BINOMIAL) || kind == GR_RANDBITS || kind == GR_SERVE_MVNORMAL;
}

}  // namespace

struct gr_server {
  int nclients = 0;
  std::vector<gr_engine*> eng;
  std::vector<gr_mvnormal*> mv;  // per client (GR_SERVE_MVNORMAL)
  int mv_dim = 0;
  Admission* adm = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  std::vector<uint64_t> slot_ticket;  // 0 = free
  std::vector<int> free_slots;
  cudaStream_t rel = nullptr;  // frees and reads
  cudaMemPool_t pool = nullptr;
  std::unordered_map<uint64_t, ServeReq> reqs;
  std::deque<uint64_t> done;  // finished, not yet reported
  uint64_t next_ticket = 1;
  size_t held = 0;
  int fail_allocs = 0;  // test hook: allocations left to fail
};

extern "C" {

double gr_server_now(void) {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

gr_status gr_server_destroy(gr_server* s) {
  if (!s) return GR_OK;
  for (cudaStream_t st : s->streams) cudaStreamSynchronize(st);
  for (auto& kv : s->reqs)
    if (kv.second.dev_out) cudaFreeAsync(kv.second.dev_out, s->rel);
  if (s->rel) cudaStreamSynchronize(s->rel);
  for (gr_mvnormal* g : s->mv) gr_mvnormal_destroy(g);
  for (gr_engine* e : s->eng) gr_engine_destroy(e);
  for (cudaEvent_t ev : s->events) cudaEventDestroy(ev);
  for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
  if (s->rel) cudaStreamDestroy(s->rel);
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s->adm;
  delete s;
  return GR_OK;
}

gr_status gr_server_create(gr_server** out, int32_t nclients, const uint64_t* seeds, size_t budget_bytes,
                           int32_t slots) {
  if (!out || !seeds || nclients < 1 || slots < 1 || budget_bytes == 0) return sfail(GR_ERR_INVALID, "bad argument");
  gr_server* s = new gr_server;
  s->nclients = nclients;
  s->adm = new Admission(nclients, budget_bytes, slots, 0.25);
  gr_status st = GR_OK;
  for (int c = 0; c < nclients && st == GR_OK; ++c) {
    gr_engine* e = nullptr;
    st = gr_engine_create(&e, seeds[c], 4, 1);
    if (st == GR_OK) {
      s->eng.push_back(e);
      st = engine_reserve(e, 128);  // segmented calls then allocate nothing
    }
  }
  int dev = 0;
  cudaGetDevice(&dev);
  for (int i = 0; i < slots && st == GR_OK; ++i) {
    cudaStream_t q = nullptr;
    cudaEvent_t ev = nullptr;
    if (cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      st = sfail(GR_ERR_CUDA, "stream / event creation");
      if (q) cudaStreamDestroy(q);
      break;
    }
    s->streams.push_back(q);
    s->events.push_back(ev);
    s->slot_ticket.push_back(0);
    s->free_slots.push_back(slots - 1 - i);
  }
  if (st == GR_OK && cudaStreamCreateWithFlags(&s->rel, cudaStreamNonBlocking) != cudaSuccess)
    st = sfail(GR_ERR_CUDA, "stream creation");
  if (st == GR_OK) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) {
      s->pool = nullptr;
      st = sfail(GR_ERR_CUDA, "memory pool creation");
    } else {
      uint64_t keep = budget_bytes;  // freed blocks stay reserved for reuse
      cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (st == GR_OK && cudaDeviceSynchronize() != cudaSuccess) st = sfail(GR_ERR_CUDA, "server set-up");
  if (st != GR_OK) {
    gr_server_destroy(s);
    return st;
  }
  *out = s;
  return GR_OK;
}

gr_status gr_server_set_mvnormal(gr_server* s, int32_t dim, const double* mean, const double* cov) {
  if (!s) return sfail(GR_ERR_INVALID, "server is NULL");
  gr_mvnormal* proto = nullptr;
  gr_status st = gr_mvnormal_create(&proto, GR_F32, dim, mean, cov, GR_MATRIX_FULL);
  if (st != GR_OK) return st;
  for (gr_mvnormal* g : s->mv) gr_mvnormal_destroy(g);
  s->mv.clear();
  for (int c = 0; c < s->nclients && st == GR_OK; ++c) {
    gr_mvnormal* g = nullptr;
    st = mvnormal_clone(proto, &g);
    if (st == GR_OK) s->mv.push_back(g);
  }
  gr_mvnormal_destroy(proto);
  s->mv_dim = st == GR_OK ? dim : 0;
  return st;
}

gr_status gr_server_submit(gr_server* s, const gr_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) return sfail(GR_ERR_INVALID, "NULL argument");
  if (r->client < 0 || r->client >= s->nclients) return sfail(GR_ERR_INVALID, "no such client");
  if (!serve_kind_ok(r->kind)) return sfail(GR_ERR_UNSUPPORTED, "kind not served");
  if (r->count == 0) return sfail(GR_ERR_INVALID, "empty request");
  ServeReq q;
  q.r = *r;
  if (q.r.arrival < 0) q.r.arrival = gr_server_now();
  if (r->kind == GR_SERVE_MVNORMAL) {
    if (!s->mv_dim) return sfail(GR_ERR_INVALID, "no MvNormalGen set (gr_server_set_mvnormal)");
    uint64_t samples = (r->count + s->mv_dim - 1) / s->mv_dim;
    while ((samples * s->mv_dim) % 8) ++samples;
    q.units = samples;
    q.gen = samples * s->mv_dim;
    q.bytes = q.gen * 4;
  } else {
    const bool is_int = r->kind == GR_POISSON || r->kind == GR_BINOMIAL || r->kind == GR_RANDBITS;
    if (is_int && r->dtype != GR_I32) return sfail(GR_ERR_INVALID, "integer kinds need GR_I32");
    if (!is_int && r->dtype != GR_F32 && r->dtype != GR_F64) return sfail(GR_ERR_INVALID, "bad dtype");
    const uint64_t P = r->dtype == GR_F32 ? 8 : 4;
    q.gen = (r->count + P - 1) / P * P;
    q.units = q.gen;
    q.bytes = q.gen * elem_bytes(r->dtype);
    // data-dependent samplers also take transient scratch (the FIFO lane
    // buffer and packet positions of a segmented call): budget 1.5x more
    const int k = r->kind;
    if (k == GR_GAMMA || k == GR_BETA || k == GR_POISSON || k == GR_BINOMIAL || k == GR_CHI_SQUARED ||
        k == GR_STUDENT_T)
      q.bytes += q.bytes + q.bytes / 2;
  }
  q.ticket = s->next_ticket++;
  if (!s->adm->submit(AdmitReq{q.ticket, r->client, q.bytes, q.r.arrival}))
    return sfail(GR_ERR_NOMEM, "request larger than the server's memory budget");
  *ticket = q.ticket;
  s->reqs.emplace(q.ticket, q);
  return GR_OK;
}

gr_status gr_server_progress(gr_server* s, gr_completion* done, size_t cap, size_t* ndone) {
  if (!s) return sfail(GR_ERR_INVALID, "server is NULL");
  // harvest
  for (size_t i = 0; i < s->streams.size(); ++i) {
    const uint64_t t = s->slot_ticket[i];
    if (!t) continue;
    const cudaError_t e = cudaEventQuery(s->events[i]);
    if (e == cudaErrorNotReady) continue;
    ServeReq& q = s->reqs[t];
    q.completed = gr_server_now();
    q.state = kDone;
    if (e != cudaSuccess) q.status = sfail(GR_ERR_CUDA, std::string("request: ") + cudaGetErrorString(e));
    if (q.cancelled) {  // its work is done: the result goes straight back
      q.status = GR_ERR_CANCELLED;
      if (q.dev_out) {
        cudaFreeAsync(q.dev_out, s->rel);
        q.dev_out = nullptr;
        s->held -= q.bytes;
      }
      s->adm->release(q.charged);
      q.charged = 0;
    }
    s->slot_ticket[i] = 0;
    s->free_slots.push_back((int)i);
    s->adm->finish(q.r.client);
    s->done.push_back(t);
  }
  // admit
  const double now = gr_server_now();
  for (const AdmitReq& a : s->adm->admit(now)) {
    ServeReq& q = s->reqs[a.ticket];
    const int slot = s->free_slots.back();
    s->free_slots.pop_back();
    cudaStream_t st = s->streams[slot];
    q.slot = slot;
    q.admitted = now;
    q.charged = q.bytes;
    gr_status rs = GR_OK;
    if (s->fail_allocs > 0) {
      --s->fail_allocs;
      q.dev_out = nullptr;
      rs = sfail(GR_ERR_NOMEM, "device memory pool exhausted (test hook)");
    } else if (cudaMallocFromPoolAsync(&q.dev_out, q.bytes, s->pool, st) != cudaSuccess) {
      cudaGetLastError();
      q.dev_out = nullptr;
      rs = sfail(GR_ERR_NOMEM, "device memory pool exhausted");
    }
    if (rs == GR_OK) {
      s->held += q.bytes;
      gr_engine* e = s->eng[q.r.client];
      if (q.r.kind == GR_SERVE_MVNORMAL) {
        rs = gr_mvnormal_sample(s->mv[q.r.client], e, q.dev_out, q.units, st);
      } else {
        gr_dist_desc d{};
        d.kind = q.r.kind;
        d.dtype = q.r.dtype;
        d.a = q.r.a;
        d.b = q.r.b;
        d.trials = q.r.trials;
        rs = gr_sample(e, &d, q.dev_out, q.units, st);
      }
    }
    if (rs == GR_OK && cudaEventRecord(s->events[slot], st) != cudaSuccess) rs = sfail(GR_ERR_CUDA, "event record");
    if (rs != GR_OK) {  // nothing was queued on the GPU for it (or only the allocation)
      q.status = rs;
      q.state = kDone;
      q.completed = gr_server_now();
      s->free_slots.push_back(slot);
      s->adm->finish(q.r.client);
      s->done.push_back(q.ticket);
      continue;
    }
    q.state = kRunning;
    s->slot_ticket[slot] = q.ticket;
  }
  // report
  size_t n = 0;
  while (n < cap && !s->done.empty() && done) {
    ServeReq& q = s->reqs[s->done.front()];
    q.reported = true;
    gr_completion& c = done[n++];
    c.ticket = q.ticket;
    c.status = q.status;
    c.client = q.r.client;
    c.dev_out = q.dev_out;
    c.count = q.gen;
    c.bytes = q.bytes;
    c.arrival = q.r.arrival;
    c.admitted = q.admitted;
    c.completed = q.completed;
    s->done.pop_front();
  }
  if (ndone) *ndone = n;
  return GR_OK;
}

gr_status gr_server_read(gr_server* s, uint64_t ticket, void* host_dst, size_t bytes) {
  if (!s || !host_dst) return sfail(GR_ERR_INVALID, "NULL argument");
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second.state != kDone || !it->second.dev_out)
    return sfail(GR_ERR_INVALID, "no finished result for this ticket");
  if (bytes > it->second.bytes) return sfail(GR_ERR_INVALID, "read beyond the result");
  SV_CUDA(cudaMemcpyAsync(host_dst, it->second.dev_out, bytes, cudaMemcpyDeviceToHost, s->rel));
  SV_CUDA(cudaStreamSynchronize(s->rel));
  return GR_OK;
}

gr_status gr_server_release(gr_server* s, uint64_t ticket) {
  if (!s) return sfail(GR_ERR_INVALID, "server is NULL");
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end() || it->second.state != kDone) return sfail(GR_ERR_INVALID, "no finished result for this ticket");
  ServeReq& q = it->second;
  if (q.dev_out) {
    SV_CUDA(cudaFreeAsync(q.dev_out, s->rel));
    s->held -= q.bytes;
  }
  s->adm->release(q.charged);
  s->reqs.erase(it);
  return GR_OK;
}

gr_status gr_server_cancel(gr_server* s, uint64_t ticket) {
  if (!s) return sfail(GR_ERR_INVALID, "server is NULL");
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(GR_ERR_INVALID, "no such ticket");
  ServeReq& q = it->second;
  if (q.state == kQueued) {
    // never admitted: nothing ran and nothing is held
    s->adm->cancel(ticket);
    q.state = kDone;
    q.status = GR_ERR_CANCELLED;
    q.completed = gr_server_now();
    s->done.push_back(ticket);
    return GR_OK;
  }
  if (q.state == kRunning) {
    q.cancelled = true;
    return GR_OK;
  }
  if (q.reported) return sfail(GR_ERR_INVALID, "the request was already reported (release it)");
  // finished, not reported yet: its result goes back now, the report says cancelled
  if (q.dev_out) {
    SV_CUDA(cudaFreeAsync(q.dev_out, s->rel));
    q.dev_out = nullptr;
    s->held -= q.bytes;
  }
  s->adm->release(q.charged);
  q.charged = 0;
  q.status = GR_ERR_CANCELLED;
  return GR_OK;
}

gr_status gr_server_cancel_client(gr_server* s, int32_t client) {
  if (!s) return sfail(GR_ERR_INVALID, "server is NULL");
  if (client < 0 || client >= s->nclients) return sfail(GR_ERR_INVALID, "no such client");
  std::vector<uint64_t> mine;
  for (const auto& kv : s->reqs)
    if (kv.second.r.client == client && !kv.second.reported && !kv.second.cancelled &&
        kv.second.status != GR_ERR_CANCELLED)
      mine.push_back(kv.first);
  std::sort(mine.begin(), mine.end());  // (admission only runs in gr_server_progress: any order would do)
  for (uint64_t t : mine) {
    const gr_status st = gr_server_cancel(s, t);
    if (st != GR_OK) return st;
  }
  return GR_OK;
}

gr_status gr_server_fail_allocs(gr_server* s, int32_t n) {
  if (!s || n < 0) return sfail(GR_ERR_INVALID, "bad argument");
  s->fail_allocs = n;
  return GR_OK;
}

gr_status gr_server_pending(const gr_server* s, size_t* queued, size_t* running, size_t* bytes_held) {
  if (!s) return sfail(GR_ERR_INVALID, "server is NULL");
  size_t r = 0;
  for (uint64_t t : s->slot_ticket) r += t ? 1 : 0;
  if (queued) *queued = s->adm->queued();
  if (running) *running = r;
  if (bytes_held) *bytes_held = s->adm->used();
  return GR_OK;
}

}  // extern "C"
