// GF(2) polynomials modulo the MT19937-64 characteristic polynomial.
#pragma once
#include <array>
#include <cstdint>
#include <vector>

namespace gr {

constexpr int kPolyDeg = 19937;
constexpr int kPolyWords = 312;  // 19968 bits
using Poly = std::array<uint64_t, kPolyWords>;

// Exponents t < 19937 with P(x) = x^19937 + sum_t x^t (empty on failure).
const std::vector<int>& charpoly_terms();
// x^e mod P(x): coefficient i is bit (i % 64) of word i / 64.
Poly pow_x_mod(uint64_t e);
// Many exponents, computed on worker threads.
void pow_x_mod_many(const std::vector<uint64_t>& exps, std::vector<Poly>& out);

}  // namespace gr
