// Pins how GCC builds a scalar engine's packets: the argument evaluation
// order of _mm256_set_epi64x / _mm256_setr_epi64x / _mm_set_epi64x with draws
// as arguments, and the words of rawbits_34 for a 64-bit engine after the
// permutevar8x32 (0,1,2,7,3,4,5,7) and shuffle_epi8 (0..11, 3, 7, 11, 11)
// that RawbitsMaker<Packet8i, Rng, uint64_t, scalar_fullbit> applies
// (arch/AVX/RandUtils.h:74-92).  Built with g++ -mavx2; prints the
// evaluation orders and 32 rawbits_34 words from std::mt19937_64(42).
#include <immintrin.h>

#include <cstdint>
#include <cstdio>
#include <random>

static uint64_t g_ctr = 0;
static uint64_t count() { return ++g_ctr; }

int main() {
  alignas(32) uint64_t e[4];
  g_ctr = 0;
  _mm256_store_si256((__m256i*)e, _mm256_set_epi64x(count(), count(), count(), count()));
  std::printf("set_epi64x %llu %llu %llu %llu\n", (unsigned long long)e[0], (unsigned long long)e[1],
              (unsigned long long)e[2], (unsigned long long)e[3]);
  g_ctr = 0;
  _mm256_store_si256((__m256i*)e, _mm256_setr_epi64x(count(), count(), count(), 0));
  std::printf("setr_epi64x %llu %llu %llu %llu\n", (unsigned long long)e[0], (unsigned long long)e[1],
              (unsigned long long)e[2], (unsigned long long)e[3]);
  g_ctr = 0;
  alignas(16) uint64_t h[2];
  _mm_store_si128((__m128i*)h, _mm_set_epi64x(count(), count()));
  std::printf("mm_set_epi64x %llu %llu\n", (unsigned long long)h[0], (unsigned long long)h[1]);

  std::mt19937_64 rng(42);
  std::printf("rawbits_34");
  for (int k = 0; k < 4; ++k) {
    __m256i p = _mm256_setr_epi64x(rng(), rng(), rng(), 0);
    p = _mm256_permutevar8x32_epi32(p, _mm256_setr_epi32(0, 1, 2, 7, 3, 4, 5, 7));
    p = _mm256_shuffle_epi8(p, _mm256_setr_epi8(0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 3, 7, 11, 11, 0, 1, 2, 3, 4,
                                                5, 6, 7, 8, 9, 10, 11, 3, 7, 11, 11));
    alignas(32) uint32_t w[8];
    _mm256_store_si256((__m256i*)w, p);
    for (int j = 0; j < 8; ++j) std::printf(" %u", w[j]);
  }
  std::printf("\n");
  return 0;
}
