// Host-only checks of the serving loop's admission policy (gr_admit.h).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../eigenrand_gb300/csrc/gr_admit.h"

using gr::AdmitReq;
using gr::Admission;

static int fails = 0;
#define CHECK(c)                                              \
  do {                                                        \
    if (!(c)) {                                               \
      std::printf("FAIL line %d: %s\n", __LINE__, #c);        \
      ++fails;                                                \
    }                                                         \
  } while (0)

static std::vector<uint64_t> tickets(const std::vector<AdmitReq>& v) {
  std::vector<uint64_t> t;
  for (auto& r : v) t.push_back(r.ticket);
  return t;
}

int main() {
  {  // slots bound concurrency; arrival order
    Admission a(4, 1000, 2, 1.0);
    for (int i = 0; i < 4; ++i) CHECK(a.submit(AdmitReq{(uint64_t)i + 1, i, 10, 0.0}));
    auto t = tickets(a.admit(0.0));
    CHECK(t.size() == 2 && t[0] == 1 && t[1] == 2);
    CHECK(a.admit(0.0).empty());
    a.finish(0);
    t = tickets(a.admit(0.0));
    CHECK(t.size() == 1 && t[0] == 3);
    CHECK(a.used() == 30);
  }
  {  // one request per client at a time, in submission order
    Admission a(2, 1000, 8, 1.0);
    a.submit(AdmitReq{1, 0, 10, 0.0});
    a.submit(AdmitReq{2, 0, 10, 0.0});
    a.submit(AdmitReq{3, 1, 10, 0.0});
    auto t = tickets(a.admit(0.0));
    CHECK(t.size() == 2 && t[0] == 1 && t[1] == 3);
    a.finish(0);
    t = tickets(a.admit(0.0));
    CHECK(t.size() == 1 && t[0] == 2);
  }
  {  // budget: a big request waits, smaller ones of other clients go ahead;
     // a client's later request never overtakes its blocked earlier one
    Admission a(3, 100, 8, 10.0);
    a.submit(AdmitReq{1, 0, 60, 0.0});
    a.submit(AdmitReq{2, 1, 60, 0.0});  // does not fit while 1 holds 60
    a.submit(AdmitReq{3, 1, 10, 0.0});  // same client as 2: must wait behind it
    a.submit(AdmitReq{4, 2, 30, 0.0});
    auto t = tickets(a.admit(0.0));
    CHECK(t.size() == 2 && t[0] == 1 && t[1] == 4);
    a.finish(0);
    CHECK(a.admit(0.0).empty());  // memory of 1 still held
    a.release(60);
    t = tickets(a.admit(0.0));
    CHECK(t.size() == 1 && t[0] == 2);
    a.finish(1);
    t = tickets(a.admit(0.0));
    CHECK(t.size() == 1 && t[0] == 3);
  }
  {  // starvation guard: after starve_s a waiting big request holds back later ones
    Admission a(3, 100, 8, 0.5);
    a.submit(AdmitReq{1, 0, 60, 0.0});
    CHECK(tickets(a.admit(0.0)).size() == 1);
    a.submit(AdmitReq{2, 1, 80, 0.1});
    a.submit(AdmitReq{3, 2, 10, 0.2});
    auto t = tickets(a.admit(0.3));  // 2 waited 0.2 s: 3 may go ahead
    CHECK(t.size() == 1 && t[0] == 3);
    a.finish(2);
    a.release(10);
    a.submit(AdmitReq{4, 2, 10, 0.4});
    t = tickets(a.admit(1.0));  // 2 waited 0.9 s > 0.5: nothing behind it starts
    CHECK(t.empty());
    a.finish(0);
    a.release(60);
    t = tickets(a.admit(1.1));
    CHECK(t.size() == 2 && t[0] == 2 && t[1] == 4);
  }
  {  // never-fitting requests and bad clients are refused at submit
    Admission a(2, 100, 1, 1.0);
    CHECK(!a.submit(AdmitReq{1, 0, 101, 0.0}));
    CHECK(!a.submit(AdmitReq{2, 5, 1, 0.0}));
    CHECK(a.queued() == 0);
  }
  {  // cancel: a queued request leaves the queue and is never admitted; the
     // client's later request then goes ahead; admitted ones are not queued
    Admission a(2, 100, 4, 1.0);
    a.submit(AdmitReq{1, 0, 10, 0.0});
    a.submit(AdmitReq{2, 0, 20, 0.0});
    a.submit(AdmitReq{3, 0, 30, 0.0});
    a.submit(AdmitReq{4, 1, 10, 0.0});
    CHECK(a.cancel(2));
    CHECK(!a.cancel(2));   // already gone
    CHECK(!a.cancel(99));  // unknown
    CHECK(a.queued() == 3);
    auto t = tickets(a.admit(0.0));
    CHECK(t.size() == 2 && t[0] == 1 && t[1] == 4);
    CHECK(!a.cancel(1));  // running: not in the queue
    CHECK(a.used() == 20);
    a.finish(0);
    t = tickets(a.admit(0.0));
    CHECK(t.size() == 1 && t[0] == 3);
    CHECK(a.used() == 50 && a.queued() == 0);
  }
  if (fails) return 1;
  std::printf("admission checks passed\n");
  return 0;
}
