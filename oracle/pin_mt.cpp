// Pins the oracle's MT19937-64 lane against an independent implementation:
// libstdc++'s std::mt19937_64, plus the C++ standard's known answer
// ([rand.predef]: the 10000th output of a default-constructed mt19937_64 is
// 9981545732273789042).  EigenRand's Vmt19937_64 lane l is exactly
// std::mt19937_64(seed + l) (PacketRandomEngine.h:230-265, 421-426).
// Exit status 0 = pinned.
#include <cstdio>
#include <random>
extern "C" {
#include "oracle.h"
}

int main() {
  int bad = 0;
  {
    or_mt64 s;
    or_mt64_seed(&s, 5489u);
    uint64_t v = 0;
    for (int i = 0; i < 10000; ++i) v = or_mt64_next(&s);
    if (v != 9981545732273789042ull) { std::printf("10000th output mismatch %llu\n", (unsigned long long)v); ++bad; }
  }
  const unsigned long long seeds[] = {0, 1, 42, 43, 44, 45, 1234, 1235, 1236, 1237, 5489, 0xffffffffffffffffull};
  for (unsigned long long sd : seeds) {
    or_mt64 s;
    or_mt64_seed(&s, sd);
    std::mt19937_64 ref(sd);
    for (int i = 0; i < 100000; ++i) {
      uint64_t a = or_mt64_next(&s), b = ref();
      if (a != b) { std::printf("seed %llu diverges at %d\n", sd, i); ++bad; break; }
    }
  }
  // packet engine: R[4k+l] = mt19937_64(seed+l)[k]
  {
    or_vmt* e = or_vmt_new(42, 4);
    std::mt19937_64 lanes[4] = {std::mt19937_64(42), std::mt19937_64(43), std::mt19937_64(44), std::mt19937_64(45)};
    uint64_t buf[4 * 1000];
    or_vmt_raw(e, buf, 1000);
    for (int k = 0; k < 1000 && !bad; ++k)
      for (int l = 0; l < 4; ++l)
        if (buf[4 * k + l] != lanes[l]()) { std::printf("packet stream mismatch k=%d l=%d\n", k, l); ++bad; break; }
    or_vmt_free(e);
  }
  std::printf(bad ? "PIN FAILED\n" : "PIN OK\n");
  return bad ? 1 : 0;
}
