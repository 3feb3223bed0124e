// Exhaustive check of the division-free quotients in gr_exact.h against the
// IEEE double division they replace.
#include <cstdio>
#include <cstring>

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
  return bad != 0;
}
