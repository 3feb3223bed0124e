// Calls the sampling library through the Eigen::Rand facade
// (include/gpurand/EigenRand.hpp) the way EigenRand code is written, and
// writes every result to a binary file for tests/test_gpu_facade.py to check
// against the CPU oracle.
//
// Record layout: u32 name length, name bytes, u32 dtype (0 f32, 1 f64, 2 i32),
// u64 element count, then the elements in Eigen's linear order.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gpurand/EigenRand.hpp"

namespace {

FILE* out = nullptr;

template <typename T>
void put(const std::string& name, const gpurand::DeviceArray<T>& m) {
  const std::vector<T> h = m.toHost();
  const uint32_t len = (uint32_t)name.size();
  const uint32_t dt = (uint32_t)gpurand::dtype_of<T>::value;
  const uint64_t n = h.size();
  fwrite(&len, 4, 1, out);
  fwrite(name.data(), 1, len, out);
  fwrite(&dt, 4, 1, out);
  fwrite(&n, 8, 1, out);
  fwrite(h.data(), sizeof(T), h.size(), out);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: facade_check OUT\n");
    return 2;
  }
  out = fopen(argv[1], "wb");
  if (!out) return 2;
  using namespace Eigen::Rand;
  try {
    // free functions on one engine, consecutive calls advance it
    Vmt19937_64 urng{42};
    gpurand::MatrixXf mf = normal<gpurand::MatrixXf>(1024, 1024, urng);
    put("normal_f32", mf);
    mf = uniformReal<gpurand::MatrixXf>(64, 32, urng);
    put("uniformReal_f32", mf);
    gpurand::MatrixXd md = normal<gpurand::MatrixXd>(128, 64, urng, 0.5, 2.0);
    put("normal2_f64", md);
    md = gammaLike(md, urng, 0.5, 1.0);
    put("gamma05_f64", md);
    gpurand::MatrixXi mi = poisson<gpurand::MatrixXi>(256, 64, urng, 4.0);
    put("poisson4_i32", mi);
    mi = binomial<gpurand::MatrixXi>(256, 64, urng, 20, 0.3);
    put("binomial20_i32", mi);
    mi = discrete<gpurand::MatrixXi>(64, 64, urng, {1.0, 2.0, 3.0, 4.0, 5.0, 6.0});
    put("discrete6_i32", mi);
    mf = beta<gpurand::MatrixXf>(64, 64, urng, 0.5f, 2.0f);
    put("beta_f32", mf);

    // generator objects keep their caches between calls
    Vmt19937_64 urng2{7};
    NormalGen<double> ng{1.0, 3.0};
    md = ng.generate<gpurand::MatrixXd>(3, 4, urng2);  // 12 = 3 packets: leaves the cos half cached
    put("normalgen_a", md);
    md = ng.generate<gpurand::MatrixXd>(5, 4, urng2);
    put("normalgen_b", md);
    GammaGen<float> gg{0.5f};
    mf = gg.generate<gpurand::MatrixXf>(8, 5, urng2);
    put("gammagen_a", mf);
    mf = gg.generateLike(mf, urng2);
    put("gammagen_b", mf);

    // P8_mt19937_64, the reference tests' engine, as the Urng
    P8_mt19937_64 p8{42};
    mf = balanced<gpurand::MatrixXf>(8, 8, p8);
    put("p8_balanced_f32", mf);
    mf = uniformReal<gpurand::MatrixXf>(8, 8, p8);
    put("p8_uniformReal_f32", mf);

    // multivariate
    Vmt19937_64 urng3{99};
    MvNormalGen<float> mv{{0.0, 1.0, -1.0, 2.0}, {4.0, 1.0, 0.5, 0.0, 1.0, 3.0, 0.2, 0.1, 0.5, 0.2, 2.0, 0.3, 0.0, 0.1, 0.3, 1.0}};
    mf = mv.generate(urng3, 1024);
    put("mvnormal_f32", mf);
    MultinomialGen<int32_t> mn{20, {0.1, 0.2, 0.3, 0.4}};
    mi = mn.generate(urng3, 64);
    put("multinomial_i32", mi);

    // errors come back as exceptions: a non-finite weight sum (AliasMethod,
    // 16 weights or more, Discrete.h:88)
    bool threw = false;
    try {
      std::vector<double> w(16, 1.0);
      w[3] = std::nan("");
      mi = discrete<gpurand::MatrixXi>(8, 1, urng3, w.begin(), w.end());
    } catch (const gpurand::Error& e) {
      threw = e.status == GR_ERR_NAN_WEIGHT || e.status == GR_ERR_INVALID;
    }
    gpurand::MatrixXi flag(1, 1);
    flag.fromHost({threw ? 1 : 0});
    put("nan_weight_threw", flag);
    urng.sync();
  } catch (const std::exception& e) {
    fprintf(stderr, "facade_check: %s\n", e.what());
    fclose(out);
    return 1;
  }
  fclose(out);
  printf("facade_check ok\n");
  return 0;
}
