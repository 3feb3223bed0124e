// Host-side check of the jump-ahead algebra used by the library: the lane
// window e words ahead equals sum_i c_i * window(i), c = x^e mod P(x).
// Compares against sequential std::mt19937_64 raw words.  Exit 0 = pass.
#include <cstdio>
#include <cstdint>
#include <vector>
#include <random>
#include "../../eigenrand_gb300/csrc/gr_poly.h"

static uint64_t tw(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t t = (a & (~0ull << 31)) | (b & ~(~0ull << 31));
  return (t >> 1) ^ ((t & 1) ? 0xb5026f5aa96619e9ull : 0) ^ c;
}

int main() {
  const auto& q = gr::charpoly_terms();
  std::printf("charpoly terms: %zu (+ x^19937)\n", q.size());
  if (q.size() != 284) return 1;
  // raw word sequence x[0..] of a lane seeded 1234
  const int total = 20600 + 70000;
  std::vector<uint64_t> x(total);
  uint64_t prev = x[0] = 1234;
  for (int i = 1; i < 312; ++i) x[i] = prev = (prev ^ (prev >> 62)) * 6364136223846793005ull + i;
  for (int i = 312; i < total; ++i) x[i] = tw(x[i - 312], x[i - 311], x[i - 156]);
  int bad = 0;
  for (uint64_t e : {1ull, 311ull, 312ull, 5000ull, 19936ull, 19937ull, 40000ull, 65536ull}) {
    if (e + 312 + 1 >= (uint64_t)total) continue;
    gr::Poly c = gr::pow_x_mod(e);
    for (int j = 1; j < 312; ++j) {  // word 0 carries only its top 33 bits
      uint64_t v = 0;
      for (int i = 0; i < 19937; ++i)
        if ((c[i / 64] >> (i % 64)) & 1) v ^= x[i + j];
      if (v != x[e + j]) { std::printf("mismatch e=%llu j=%d\n", (unsigned long long)e, j); ++bad; break; }
    }
    uint64_t v0 = 0;
    for (int i = 0; i < 19937; ++i)
      if ((c[i / 64] >> (i % 64)) & 1) v0 ^= x[i];
    if ((v0 ^ x[e]) & (~0ull << 31)) { std::printf("top bits mismatch e=%llu\n", (unsigned long long)e); ++bad; }
  }
  std::printf(bad ? "JUMP FAILED\n" : "JUMP OK\n");
  return bad ? 1 : 0;
}
