// Admission policy of the serving loop (host only, no CUDA).
//
// Requests queue in arrival order.  One pass of admit() starts, in that
// order, every request whose client has nothing running or queued ahead of
// it (a client's engine is sequential, so its requests run one at a time and
// in order), whose output fits in what is left of the device-memory budget,
// while stream slots are free.  A request that does not fit is skipped
// (later, smaller requests of other clients go ahead) until it has waited
// longer than starve_s; from then on nothing behind it is admitted until it
// fits.  Memory is held from admission until the caller releases the result.
#pragma once
#include <cstddef>
#include <cstdint>
#include <list>
#include <vector>

namespace gr {

struct AdmitReq {
  uint64_t ticket;
  int client;
  size_t bytes;
  double arrival;  // seconds
};

class Admission {
 public:
  Admission(int nclients, size_t budget, int slots, double starve_s)
      : busy_(nclients, 0), budget_(budget), free_slots_(slots), starve_s_(starve_s) {}

  // false when the request can never fit (bytes > budget) or names no client
  bool submit(const AdmitReq& r) {
    if (r.client < 0 || r.client >= (int)busy_.size() || r.bytes > budget_) return false;
    queue_.push_back(r);
    return true;
  }

  std::vector<AdmitReq> admit(double now) {
    std::vector<AdmitReq> out;
    std::vector<char> blocked(busy_.size(), 0);
    for (auto it = queue_.begin(); it != queue_.end() && free_slots_ > 0;) {
      const AdmitReq& r = *it;
      if (busy_[r.client] || blocked[r.client]) {
        blocked[r.client] = 1;
        ++it;
        continue;
      }
      if (used_ + r.bytes > budget_) {
        blocked[r.client] = 1;
        if (now - r.arrival > starve_s_) break;  // hold everything behind it back
        ++it;
        continue;
      }
      used_ += r.bytes;
      busy_[r.client] = 1;
      --free_slots_;
      out.push_back(r);
      it = queue_.erase(it);
    }
    return out;
  }

  // drops a queued (not yet admitted) request; false if it is not queued
  bool cancel(uint64_t ticket) {
    for (auto it = queue_.begin(); it != queue_.end(); ++it)
      if (it->ticket == ticket) {
        queue_.erase(it);
        return true;
      }
    return false;
  }

  // the request's GPU work is done: its slot and its client are free again
  void finish(int client) {
    busy_[client] = 0;
    ++free_slots_;
  }
  // the request's memory is given back
  void release(size_t bytes) { used_ = bytes > used_ ? 0 : used_ - bytes; }

  size_t used() const { return used_; }
  size_t budget() const { return budget_; }
  int free_slots() const { return free_slots_; }
  size_t queued() const { return queue_.size(); }

 private:
  std::list<AdmitReq> queue_;
  std::vector<char> busy_;
  size_t budget_;
  size_t used_ = 0;
  int free_slots_;
  double starve_s_;
};

}  // namespace gr
