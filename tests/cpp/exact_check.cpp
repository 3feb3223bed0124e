// Exhaustive check of the division-free quotients in gr_exact.h against the
// IEEE double division they replace.
#include <cstdio>
#include <cstring>
#include <initializer_list>

#include "gr_exact.h"

int main() {
  unsigned long long bad = 0;
  for (unsigned long long k = 0; k <= 0x7fffffffull; ++k) {
    const double want = (double)(int)k / 2147483647.0, got = gr::div_2p31m1((uint32_t)k);
    if (std::memcmp(&want, &got, sizeof want) != 0) {
      if (bad < 5) std::printf("k=%llu want %a got %a\n", k, want, got);
      ++bad;
    }
  }
  std::printf("div_2p31m1 mismatches %llu of 2^31\n", bad);
  // one_minus_ur_d: every fraction near both ends, and a stride through the rest
  unsigned long long bad2 = 0, cnt = 0;
  auto check = [&](uint64_t F) {
    for (uint64_t hi : {0ull, 0x3ff0000000000000ull, 0xfff0000000000000ull}) {
      const uint64_t x = hi | F;
      const double u = gr::bits_to_double((x & 0xfffffffffffffull) | 0x3ff0000000000000ull) - 1.0;
      const double want = 1.0 - u, got = gr::one_minus_ur_d(x);
      ++cnt;
      if (std::memcmp(&want, &got, sizeof want) != 0) {
        if (bad2 < 5) std::printf("F=%llx want %a got %a\n", (unsigned long long)F, want, got);
        ++bad2;
      }
    }
  };
  for (uint64_t F = 0; F < (1ull << 22); ++F) check(F);
  for (uint64_t F = (1ull << 52) - (1ull << 22); F < (1ull << 52); ++F) check(F);
  for (uint64_t F = 0; F < (1ull << 52); F += 0x3b9aca07ull) check(F);
  std::printf("one_minus_ur_d mismatches %llu of %llu\n", bad2, cnt);
  // untempering inverts tempering (xorshift-64 sequence of inputs)
  unsigned long long bad3 = 0;
  uint64_t s = 0x9e3779b97f4a7c15ull;
  for (int i = 0; i < (1 << 24); ++i) {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    if (gr::mt_untemper64(gr::mt_temper64(s)) != s || gr::mt_temper64(gr::mt_untemper64(s)) != s) ++bad3;
  }
  std::printf("untemper mismatches %llu\n", bad3);
  // untwisting a block: twist random blocks forward, then recover each
  // previous block from the next one
  unsigned long long bad4 = 0;
  {
    uint64_t st[4][312];
    for (int b = 0; b < 4; ++b)
      for (int i = 0; i < 312; ++i) {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        st[b][i] = s;
      }
    for (int rep = 0; rep < 200; ++rep) {
      uint64_t old[312], nw[312], back[312];
      for (int i = 0; i < 312; ++i) old[i] = st[rep % 4][(i + rep) % 312] ^ (uint64_t)rep * 0x9e3779b97f4a7c15ull;
      auto f = [](uint64_t y) { return (y >> 1) ^ ((y & 1) ? 0xb5026f5aa96619e9ull : 0ull); };
      for (int i = 0; i < 312; ++i) {
        const uint64_t nxt = i + 1 < 312 ? old[i + 1] : nw[0];
        const uint64_t y = (old[i] & 0xffffffff80000000ull) | (nxt & 0x000000007fffffffull);
        nw[i] = (i < 156 ? old[i + 156] : nw[i - 156]) ^ f(y);
      }
      // old[0]'s lower bits only matter through old[311] = old[155] ^ f(...):
      // make the pair consistent, as any block produced by a twist is
      const uint64_t y311 = (0ull) | (old[0] & 0x000000007fffffffull);
      old[311] = old[155] ^ f(y311);
      for (int i = 0; i < 312; ++i) {
        const uint64_t nxt = i + 1 < 312 ? old[i + 1] : nw[0];
        const uint64_t y = (old[i] & 0xffffffff80000000ull) | (nxt & 0x000000007fffffffull);
        nw[i] = (i < 156 ? old[i + 156] : nw[i - 156]) ^ f(y);
      }
      for (int i = 0; i < 312; ++i) back[i] = 0x5555555555555555ull;
      gr::mt_untwist_block([&](int i) -> uint64_t& { return nw[i]; }, [&](int i) -> uint64_t& { return back[i]; });
      for (int i = 0; i < 312; ++i) bad4 += back[i] != old[i];
    }
  }
  std::printf("untwist mismatches %llu\n", bad4);
  return bad != 0 || bad2 != 0 || bad3 != 0 || bad4 != 0;
}
