// GF(2) polynomial arithmetic for MT19937-64 jump-ahead (host side).
//
// The characteristic polynomial P(x) of the MT19937-64 state transition
// (degree 19937) is recovered once per process with the Berlekamp-Massey
// algorithm from the low bit of 2*19937+64 outputs of std::mt19937_64 (the
// exact lane generator of Vmt19937_64, PacketRandomEngine.h:421-426).  It has
// 285 non-zero terms, so reduction modulo P is cheap and x^e mod P follows by
// square-and-multiply-by-x (Haramoto, Matsumoto, L'Ecuyer, "A Fast Jump Ahead
// Algorithm for Linear Recurrences in a Polynomial Space", 2008).
#include "gr_poly.h"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <random>
#include <thread>

namespace gr {
namespace {

std::vector<int> compute_charpoly_terms() {
  const int M = 2 * kPolyDeg + 64;
  std::vector<uint8_t> s(M);
  std::mt19937_64 g(5489u);
  for (int i = 0; i < M; ++i) s[i] = (uint8_t)(g() & 1u);
  const int W = M / 64 + 2;
  std::vector<uint64_t> C(W, 0), B(W, 0), T(W, 0), R(W, 0);
  C[0] = 1;
  B[0] = 1;
  int L = 0, m = 1;
  for (int n = 0; n < M; ++n) {
    // R: bit i = s[n - i]
    for (int w = W - 1; w > 0; --w) R[w] = (R[w] << 1) | (R[w - 1] >> 63);
    R[0] = (R[0] << 1) | s[n];
    const int lw = L / 64 + 1;
    uint64_t acc = 0;
    for (int w = 0; w < lw && w < W; ++w) acc ^= C[w] & R[w];
    // bits of C above L are zero, so the tail words contribute nothing
    int d = __builtin_parityll(acc);
    if (!d) {
      ++m;
      continue;
    }
    T = C;
    // C ^= B << m
    const int ws = m / 64, bs = m % 64;
    for (int w = W - 1; w >= ws; --w) {
      uint64_t v = B[w - ws] << bs;
      if (bs && w - ws - 1 >= 0) v |= B[w - ws - 1] >> (64 - bs);
      C[w] ^= v;
    }
    if (2 * L <= n) {
      L = n + 1 - L;
      B = T;
      m = 1;
    } else {
      ++m;
    }
  }
  std::vector<int> terms;  // exponents t < deg of P(x) - x^deg
  if (L != kPolyDeg) return terms;
  for (int i = 1; i <= L; ++i)
    if ((C[i / 64] >> (i % 64)) & 1u) terms.push_back(L - i);
  std::sort(terms.begin(), terms.end());
  return terms;
}

inline void xor_shifted(uint64_t* v, int nwords, uint64_t h, int pos) {
  // v ^= h * x^pos  (pos >= 0)
  const int w = pos >> 6, b = pos & 63;
  if (w < nwords) v[w] ^= h << b;
  if (b && w + 1 < nwords) v[w + 1] ^= h >> (64 - b);
}

// reduce v (2*kPolyWords words) modulo P into its low kPolyWords words
void reduce(uint64_t* v, const std::vector<int>& q) {
  const int top = 2 * kPolyWords - 1;
  const int bw = kPolyDeg / 64;        // 311: word holding bit kPolyDeg
  const int bb = kPolyDeg % 64;        // 33
  for (int w = top; w >= bw; --w) {
    for (;;) {
      uint64_t h = v[w];
      if (w == bw) h &= ~((1ull << bb) - 1);
      if (!h) break;
      v[w] ^= h;
      // bit (64w + b) -> x^(64w + b - deg) * Q(x)
      if (w == bw) {
        const uint64_t h2 = h >> bb;  // bits >= deg, now at offset 0
        for (int t : q) xor_shifted(v, 2 * kPolyWords, h2, t);
      } else {
        const int base = 64 * w - kPolyDeg;
        for (int t : q) xor_shifted(v, 2 * kPolyWords, h, base + t);
      }
    }
  }
}

inline uint64_t spread32(uint32_t x) {
  uint64_t v = x;
  v = (v | (v << 16)) & 0x0000ffff0000ffffull;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}

void sqr_mod(Poly& a, const std::vector<int>& q) {
  uint64_t v[2 * kPolyWords];
  for (int w = 0; w < kPolyWords; ++w) {
    v[2 * w] = spread32((uint32_t)a[w]);
    v[2 * w + 1] = spread32((uint32_t)(a[w] >> 32));
  }
  reduce(v, q);
  std::memcpy(a.data(), v, sizeof(uint64_t) * kPolyWords);
}

void mulx_mod(Poly& a, const std::vector<int>& q) {
  const int bw = kPolyDeg / 64, bb = kPolyDeg % 64;
  for (int w = kPolyWords - 1; w > 0; --w) a[w] = (a[w] << 1) | (a[w - 1] >> 63);
  a[0] <<= 1;
  if ((a[bw] >> bb) & 1u) {
    a[bw] ^= 1ull << bb;
    for (int t : q) a[t >> 6] ^= 1ull << (t & 63);
  }
}

}  // namespace

const std::vector<int>& charpoly_terms() {
  static std::once_flag once;
  static std::vector<int> terms;
  std::call_once(once, [] { terms = compute_charpoly_terms(); });
  return terms;
}

Poly pow_x_mod(uint64_t e) {
  const std::vector<int>& q = charpoly_terms();
  Poly r{};
  r[0] = 1;
  if (e == 0) return r;
  int top = 63;
  while (!((e >> top) & 1u)) --top;
  for (int b = top; b >= 0; --b) {
    sqr_mod(r, q);
    if ((e >> b) & 1u) mulx_mod(r, q);
  }
  return r;
}

void pow_x_mod_many(const std::vector<uint64_t>& exps, std::vector<Poly>& out) {
  out.assign(exps.size(), Poly{});
  charpoly_terms();
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  nt = std::min<unsigned>(nt, (unsigned)std::max<size_t>(1, exps.size()));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    th.emplace_back([&, t] {
      for (size_t i = t; i < exps.size(); i += nt) out[i] = pow_x_mod(exps[i]);
    });
  }
  for (auto& x : th) x.join();
}

}  // namespace gr
