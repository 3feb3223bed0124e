/*
 * EigenRand.hpp — the Eigen::Rand call surface over the C ABI (gpurand.h).
 *
 * Header-only C++17.  Code written against EigenRand's free functions and
 * generator classes (bab2min/EigenRand v0.6.0: the headers under
 * EigenRand/Dists and EigenRand/MvDists) keeps its names, parameter order and defaults:
 *
 *     Eigen::Rand::Vmt19937_64 urng{ 42 };
 *     gpurand::MatrixXf m = Eigen::Rand::normal<gpurand::MatrixXf>(1024, 1024, urng);
 *     Eigen::Rand::GammaGen<float> gen{ 0.5f };
 *     m = gen.generate<gpurand::MatrixXf>(1024, 1024, urng);
 *
 * What changes is where the numbers live.  The reference returns a lazy Eigen
 * expression that is evaluated when it is assigned into caller-owned host
 * storage; here the expression is evaluated when it is assigned into a
 * gpurand::DeviceArray<T> (column-major, device memory, Eigen's linear
 * order), on the engine's CUDA stream, by the library's kernels.  The
 * samples are the reference's: bit-exact for the engine streams and the
 * integer kinds, and as documented in gpurand.h for the rest.
 *
 * Engines are captured by reference, so each call advances the caller's
 * engine, as the reference's lvalue engines do (RandUtils.h:67-72).  A
 * generator object keeps its caches between calls (StdNormalGen's cached
 * half, CompressMask's carried lanes).  Errors are thrown as
 * gpurand::Error (the reference throws std::invalid_argument / asserts).
 *
 * Link with libgpurand.so and the CUDA runtime (-lcudart).
 */
#ifndef GPURAND_EIGENRAND_HPP
#define GPURAND_EIGENRAND_HPP

#include <cuda_runtime_api.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../gpurand.h"

namespace gpurand {

using Index = std::ptrdiff_t;

class Error : public std::runtime_error {
 public:
  Error(gr_status s, const std::string& where)
      : std::runtime_error(where + ": " + (gr_last_error() ? gr_last_error() : "")), status(s) {}
  gr_status status;
};

inline void check(gr_status s, const char* where) {
  if (s != GR_OK) throw Error(s, where);
}
inline void check_cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
struct dtype_of;
template <>
struct dtype_of<float> {
  static constexpr int32_t value = GR_F32;
};
template <>
struct dtype_of<double> {
  static constexpr int32_t value = GR_F64;
};
template <>
struct dtype_of<int32_t> {
  static constexpr int32_t value = GR_I32;
};

// A dense column-major array in device memory: the storage a random
// expression is assigned into (the role Eigen::Matrix / Array play).
template <typename T>
class DeviceArray {
 public:
  using Scalar = T;
  DeviceArray() = default;
  DeviceArray(Index rows, Index cols) { resize(rows, cols); }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept { swap(o); }
  DeviceArray& operator=(DeviceArray&& o) noexcept {
    swap(o);
    return *this;
  }
  ~DeviceArray() {
    if (data_) cudaFree(data_);
  }
  // evaluates a random expression into this array (see below)
  template <typename Expr, typename = decltype(std::declval<const Expr&>().evalTo(std::declval<DeviceArray&>()))>
  DeviceArray(const Expr& e) {
    e.evalTo(*this);
  }
  template <typename Expr, typename = decltype(std::declval<const Expr&>().evalTo(std::declval<DeviceArray&>()))>
  DeviceArray& operator=(const Expr& e) {
    e.evalTo(*this);
    return *this;
  }
  void resize(Index rows, Index cols) {
    if (rows * cols != rows_ * cols_) {
      if (data_) cudaFree(data_);
      data_ = nullptr;
      if (rows * cols > 0) check_cuda(cudaMalloc(reinterpret_cast<void**>(&data_), sizeof(T) * rows * cols), "cudaMalloc");
    }
    rows_ = rows;
    cols_ = cols;
  }
  Index rows() const { return rows_; }
  Index cols() const { return cols_; }
  Index size() const { return rows_ * cols_; }
  T* data() { return data_; }
  const T* data() const { return data_; }
  // Eigen's linear (column-major) order
  std::vector<T> toHost() const {
    std::vector<T> h((size_t)size());
    if (size()) check_cuda(cudaMemcpy(h.data(), data_, sizeof(T) * size(), cudaMemcpyDeviceToHost), "cudaMemcpy");
    return h;
  }
  void fromHost(const std::vector<T>& h) {
    if ((Index)h.size() != size()) throw std::invalid_argument("fromHost: size mismatch");
    if (size()) check_cuda(cudaMemcpy(data_, h.data(), sizeof(T) * size(), cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  void swap(DeviceArray& o) noexcept {
    std::swap(data_, o.data_);
    std::swap(rows_, o.rows_);
    std::swap(cols_, o.cols_);
  }

 private:
  T* data_ = nullptr;
  Index rows_ = 0, cols_ = 0;
};

using MatrixXf = DeviceArray<float>;
using MatrixXd = DeviceArray<double>;
using MatrixXi = DeviceArray<int32_t>;
using ArrayXXf = DeviceArray<float>;
using ArrayXXd = DeviceArray<double>;
using ArrayXXi = DeviceArray<int32_t>;

namespace detail {
inline gr_dist_desc desc(int32_t kind, int32_t dtype, double a = 0, double b = 0, int32_t trials = 0) {
  gr_dist_desc d{};
  d.kind = kind;
  d.dtype = dtype;
  d.a = a;
  d.b = b;
  d.trials = trials;
  return d;
}
}  // namespace detail

}  // namespace gpurand

namespace Eigen {
namespace Rand {

using gpurand::Index;

// ---- engines -----------------------------------------------------------------
// Vmt19937_64 (PacketRandomEngine.h:585-599): lanes seed + l.  streams = K
// makes K independent engines seeded seed + 4k that split every call into K
// contiguous slices (one engine per thread in the reference's usage).
class Vmt19937_64 {
 public:
  using result_type = uint64_t;
  explicit Vmt19937_64(uint64_t seed = 5489, int32_t streams = 1, cudaStream_t stream = nullptr)
      : stream_(stream) {
    gpurand::check(gr_engine_create(&e_, seed, 4, streams), "Vmt19937_64");
  }
  Vmt19937_64(const Vmt19937_64&) = delete;
  Vmt19937_64& operator=(const Vmt19937_64&) = delete;
  ~Vmt19937_64() {
    if (e_) gr_engine_destroy(e_);
  }
  void seed(uint64_t s) { gpurand::check(gr_engine_seed(e_, s, stream()), "seed"); }
  void discard(unsigned long long num) { gpurand::check(gr_engine_discard(e_, num, stream()), "discard"); }
  // waits for the engine's work and reports device-side errors
  void sync() { gpurand::check(gr_engine_sync(e_, stream()), "sync"); }
  gr_engine* handle() const { return e_; }
  gr_stream_t stream() const { return reinterpret_cast<gr_stream_t>(stream_); }

 private:
  gr_engine* e_ = nullptr;
  cudaStream_t stream_ = nullptr;
};

// Scalar 64-bit engines as the Urng (RandomEngineType::scalar_fullbit):
// std::mt19937_64 and P8_mt19937_64 (PacketRandomEngine.h:600-607).
template <int32_t KIND>
class ScalarEngine {
 public:
  using result_type = uint64_t;
  explicit ScalarEngine(uint64_t seed = 5489, cudaStream_t stream = nullptr) : stream_(stream) {
    gpurand::check(gr_sengine_create(&e_, KIND, seed), "scalar engine");
  }
  ScalarEngine(const ScalarEngine&) = delete;
  ScalarEngine& operator=(const ScalarEngine&) = delete;
  ~ScalarEngine() {
    if (e_) gr_sengine_destroy(e_);
  }
  gr_sengine* handle() const { return e_; }
  gr_stream_t stream() const { return reinterpret_cast<gr_stream_t>(stream_); }

 private:
  gr_sengine* e_ = nullptr;
  cudaStream_t stream_ = nullptr;
};
using P8_mt19937_64 = ScalarEngine<GR_SCALAR_P8_MT19937_64>;
// std::mt19937_64 as the Urng, device resident (same stream as std::mt19937_64)
using Mt19937_64 = ScalarEngine<GR_SCALAR_MT19937_64>;

namespace detail {
inline void sample(Vmt19937_64& u, const gr_dist_desc& d, void* out, size_t n) {
  gpurand::check(gr_sample(u.handle(), &d, out, n, u.stream()), "sample");
}
template <int32_t K>
inline void sample(ScalarEngine<K>& u, const gr_dist_desc& d, void* out, size_t n) {
  gpurand::check(gr_sengine_sample(u.handle(), &d, out, n, u.stream()), "sample");
}
}  // namespace detail

// ---- random expressions --------------------------------------------------------
// What a free function returns: the shape, the engine (by reference) and the
// distribution.  Assigning it into a DeviceArray draws the samples.
template <typename Derived, typename Urng>
class RandExpr {
 public:
  using Scalar = typename Derived::Scalar;
  RandExpr(Index rows, Index cols, Urng& urng, const gr_dist_desc& d, std::vector<double> w = {})
      : rows_(rows), cols_(cols), urng_(urng), d_(d), w_(std::move(w)) {}
  Index rows() const { return rows_; }
  Index cols() const { return cols_; }
  void evalTo(gpurand::DeviceArray<Scalar>& dst) const {
    dst.resize(rows_, cols_);
    gr_dist_desc d = d_;
    if (!w_.empty()) {
      d.weights = w_.data();
      d.nweights = (int32_t)w_.size();
    }
    detail::sample(urng_, d, dst.data(), (size_t)(rows_ * cols_));
  }
  Derived eval() const {
    Derived m;
    evalTo(m);
    return m;
  }

 private:
  Index rows_, cols_;
  Urng& urng_;
  gr_dist_desc d_;
  std::vector<double> w_;
};

// ---- generator classes (Dists/*.h) ---------------------------------------------
// One generator object; generate / generateLike (Basic.h:34-79) draw with its
// caches, carried between calls.  Packet engines only (Vmt19937_64); with a
// scalar engine use the free functions, as the reference's cached generators
// are tied to packet draws.
template <typename Scalar>
class GenBase {
 public:
  GenBase(const GenBase&) = delete;
  GenBase& operator=(const GenBase&) = delete;
  ~GenBase() {
    if (g_) gr_gen_destroy(g_);
  }
  gr_gen* handle() const { return g_; }

 protected:
  explicit GenBase(const gr_dist_desc& d) { gpurand::check(gr_gen_create(&g_, &d), "generator"); }
  gr_gen* g_ = nullptr;
};

template <typename Derived, typename Gen>
class GenExpr {
 public:
  using Scalar = typename Derived::Scalar;
  GenExpr(Index rows, Index cols, Vmt19937_64& urng, const Gen& g) : rows_(rows), cols_(cols), urng_(urng), g_(g) {}
  void evalTo(gpurand::DeviceArray<Scalar>& dst) const {
    dst.resize(rows_, cols_);
    gpurand::check(gr_generate(g_.handle(), urng_.handle(), dst.data(), (size_t)(rows_ * cols_), urng_.stream()),
                   "generate");
  }
  Derived eval() const {
    Derived m;
    evalTo(m);
    return m;
  }

 private:
  Index rows_, cols_;
  Vmt19937_64& urng_;
  const Gen& g_;
};

#define GPURAND_GEN_COMMON(NAME)                                                    \
  template <typename Derived>                                                       \
  GenExpr<Derived, NAME> generate(Index rows, Index cols, Vmt19937_64& urng) const { \
    return {rows, cols, urng, *this};                                               \
  }                                                                                 \
  template <typename Derived>                                                       \
  GenExpr<Derived, NAME> generateLike(const Derived& o, Vmt19937_64& urng) const {  \
    return {o.rows(), o.cols(), urng, *this};                                       \
  }

template <typename _Scalar>
class StdUniformRealGen : public GenBase<_Scalar> {
 public:
  StdUniformRealGen() : GenBase<_Scalar>(gpurand::detail::desc(GR_UNIFORM_REAL, gpurand::dtype_of<_Scalar>::value)) {}
  GPURAND_GEN_COMMON(StdUniformRealGen)
};
template <typename _Scalar>
class UniformRealGen : public GenBase<_Scalar> {
 public:
  UniformRealGen(_Scalar min = 0, _Scalar max = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_UNIFORM_REAL2, gpurand::dtype_of<_Scalar>::value, min, max)) {}
  GPURAND_GEN_COMMON(UniformRealGen)
};
template <typename _Scalar>
class BalancedGen : public GenBase<_Scalar> {
 public:
  BalancedGen() : GenBase<_Scalar>(gpurand::detail::desc(GR_BALANCED, gpurand::dtype_of<_Scalar>::value)) {}
  GPURAND_GEN_COMMON(BalancedGen)
};
template <typename _Scalar>
class Balanced2Gen : public GenBase<_Scalar> {
 public:
  Balanced2Gen(_Scalar a = -1, _Scalar b = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_BALANCED2, gpurand::dtype_of<_Scalar>::value, a, b)) {}
  GPURAND_GEN_COMMON(Balanced2Gen)
};
template <typename _Scalar>
class StdNormalGen : public GenBase<_Scalar> {
 public:
  StdNormalGen() : GenBase<_Scalar>(gpurand::detail::desc(GR_NORMAL_STD, gpurand::dtype_of<_Scalar>::value)) {}
  GPURAND_GEN_COMMON(StdNormalGen)
};
template <typename _Scalar>
class NormalGen : public GenBase<_Scalar> {
 public:
  NormalGen(_Scalar mean = 0, _Scalar stdev = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_NORMAL, gpurand::dtype_of<_Scalar>::value, mean, stdev)) {}
  GPURAND_GEN_COMMON(NormalGen)
};
template <typename _Scalar>
class LognormalGen : public GenBase<_Scalar> {
 public:
  LognormalGen(_Scalar mean = 0, _Scalar stdev = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_LOGNORMAL, gpurand::dtype_of<_Scalar>::value, mean, stdev)) {}
  GPURAND_GEN_COMMON(LognormalGen)
};
template <typename _Scalar>
class ExponentialGen : public GenBase<_Scalar> {
 public:
  ExponentialGen(_Scalar lambda = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_EXPONENTIAL, gpurand::dtype_of<_Scalar>::value, lambda)) {}
  GPURAND_GEN_COMMON(ExponentialGen)
};
template <typename _Scalar>
class CauchyGen : public GenBase<_Scalar> {
 public:
  CauchyGen(_Scalar a = 0, _Scalar b = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_CAUCHY, gpurand::dtype_of<_Scalar>::value, a, b)) {}
  GPURAND_GEN_COMMON(CauchyGen)
};
template <typename _Scalar>
class WeibullGen : public GenBase<_Scalar> {
 public:
  WeibullGen(_Scalar a = 1, _Scalar b = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_WEIBULL, gpurand::dtype_of<_Scalar>::value, a, b)) {}
  GPURAND_GEN_COMMON(WeibullGen)
};
template <typename _Scalar>
class ExtremeValueGen : public GenBase<_Scalar> {
 public:
  ExtremeValueGen(_Scalar a = 0, _Scalar b = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_EXTREME_VALUE, gpurand::dtype_of<_Scalar>::value, a, b)) {}
  GPURAND_GEN_COMMON(ExtremeValueGen)
};
template <typename _Scalar>
class GammaGen : public GenBase<_Scalar> {
 public:
  GammaGen(_Scalar alpha = 1, _Scalar beta = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_GAMMA, gpurand::dtype_of<_Scalar>::value, alpha, beta)) {}
  GPURAND_GEN_COMMON(GammaGen)
};
template <typename _Scalar>
class BetaGen : public GenBase<_Scalar> {
 public:
  BetaGen(_Scalar a = 1, _Scalar b = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_BETA, gpurand::dtype_of<_Scalar>::value, a, b)) {}
  GPURAND_GEN_COMMON(BetaGen)
};
template <typename _Scalar>
class StudentTGen : public GenBase<_Scalar> {
 public:
  StudentTGen(_Scalar n = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_STUDENT_T, gpurand::dtype_of<_Scalar>::value, n)) {}
  GPURAND_GEN_COMMON(StudentTGen)
};
template <typename _Scalar>
class ChiSquaredGen : public GenBase<_Scalar> {
 public:
  ChiSquaredGen(_Scalar n = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_CHI_SQUARED, gpurand::dtype_of<_Scalar>::value, n)) {}
  GPURAND_GEN_COMMON(ChiSquaredGen)
};
template <typename _Scalar>
class FisherFGen : public GenBase<_Scalar> {
 public:
  FisherFGen(_Scalar m = 1, _Scalar n = 1)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_FISHER_F, gpurand::dtype_of<_Scalar>::value, m, n)) {}
  GPURAND_GEN_COMMON(FisherFGen)
};
template <typename _Scalar>
class BernoulliGen : public GenBase<_Scalar> {
 public:
  BernoulliGen(double p = 0.5)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_BERNOULLI, gpurand::dtype_of<_Scalar>::value, p)) {}
  GPURAND_GEN_COMMON(BernoulliGen)
};
template <typename _Scalar>
class RandbitsGen : public GenBase<_Scalar> {
  static_assert(std::is_same<_Scalar, int32_t>::value, "RandbitsGen: int32_t only");

 public:
  RandbitsGen() : GenBase<_Scalar>(gpurand::detail::desc(GR_RANDBITS, GR_I32)) {}
  GPURAND_GEN_COMMON(RandbitsGen)
};
template <typename _Scalar>
class UniformIntGen : public GenBase<_Scalar> {
 public:
  UniformIntGen(_Scalar min = 0, _Scalar max = 0)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_UNIFORM_INT, GR_I32, min, max)) {}
  GPURAND_GEN_COMMON(UniformIntGen)
};
template <typename _Scalar>
class PoissonGen : public GenBase<_Scalar> {
 public:
  PoissonGen(double mean = 1) : GenBase<_Scalar>(gpurand::detail::desc(GR_POISSON, GR_I32, mean)) {}
  GPURAND_GEN_COMMON(PoissonGen)
};
template <typename _Scalar>
class BinomialGen : public GenBase<_Scalar> {
 public:
  BinomialGen(_Scalar trials = 1, double p = 0.5)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_BINOMIAL, GR_I32, p, 0, trials)) {}
  GPURAND_GEN_COMMON(BinomialGen)
};
template <typename _Scalar>
class GeometricGen : public GenBase<_Scalar> {
 public:
  GeometricGen(double p = 0.5) : GenBase<_Scalar>(gpurand::detail::desc(GR_GEOMETRIC, GR_I32, p)) {}
  GPURAND_GEN_COMMON(GeometricGen)
};
template <typename _Scalar>
class NegativeBinomialGen : public GenBase<_Scalar> {
 public:
  NegativeBinomialGen(_Scalar trials = 1, double p = 0.5)
      : GenBase<_Scalar>(gpurand::detail::desc(GR_NEGATIVE_BINOMIAL, GR_I32, p, 0, trials)) {}
  GPURAND_GEN_COMMON(NegativeBinomialGen)
};
// DiscreteGen<int32_t, int32_t> over weights (Discrete.h:352-486)
template <typename _Scalar, typename Precision = int32_t>
class DiscreteGen : public GenBase<_Scalar> {
 public:
  template <typename It>
  DiscreteGen(It first, It last) : DiscreteGen(std::vector<double>(first, last)) {}
  DiscreteGen(std::initializer_list<double> w) : DiscreteGen(std::vector<double>(w)) {}
  explicit DiscreteGen(const std::vector<double>& w) : GenBase<_Scalar>(make(w)) {}
  GPURAND_GEN_COMMON(DiscreteGen)

 private:
  static gr_dist_desc make(const std::vector<double>& w) {
    gr_dist_desc d = gpurand::detail::desc(GR_DISCRETE, GR_I32);
    d.weights = w.data();
    d.nweights = (int32_t)w.size();
    return d;
  }
};
#undef GPURAND_GEN_COMMON

// ---- free functions (Dists/Basic.h, NormalExp.h, Discrete.h) ------------------
// rows x cols, or the shape of `o` (*Like), with the reference's defaults.
#define GPURAND_FREE0(NAME, KIND)                                                                      \
  template <typename Derived, typename Urng>                                                           \
  inline RandExpr<Derived, Urng> NAME(Index rows, Index cols, Urng& urng) {                            \
    return {rows, cols, urng, gpurand::detail::desc(KIND, gpurand::dtype_of<typename Derived::Scalar>::value)}; \
  }                                                                                                    \
  template <typename Derived, typename Urng>                                                           \
  inline RandExpr<Derived, Urng> NAME##Like(const Derived& o, Urng& urng) {                            \
    return NAME<Derived>(o.rows(), o.cols(), urng);                                                    \
  }
#define GPURAND_FREE2(NAME, KIND, DA, DB)                                                                       \
  template <typename Derived, typename Urng>                                                                    \
  inline RandExpr<Derived, Urng> NAME(Index rows, Index cols, Urng& urng, typename Derived::Scalar a = DA,      \
                                      typename Derived::Scalar b = DB) {                                        \
    return {rows, cols, urng, gpurand::detail::desc(KIND, gpurand::dtype_of<typename Derived::Scalar>::value, a, b)}; \
  }                                                                                                             \
  template <typename Derived, typename Urng>                                                                    \
  inline RandExpr<Derived, Urng> NAME##Like(const Derived& o, Urng& urng, typename Derived::Scalar a = DA,      \
                                            typename Derived::Scalar b = DB) {                                  \
    return NAME<Derived>(o.rows(), o.cols(), urng, a, b);                                                       \
  }

GPURAND_FREE0(uniformReal, GR_UNIFORM_REAL)  // Basic.h:951-1017
GPURAND_FREE0(balanced, GR_BALANCED)         // Basic.h:818-884
GPURAND_FREE0(randBits, GR_RANDBITS)         // Basic.h:786-811
GPURAND_FREE2(lognormal, GR_LOGNORMAL, 0, 1)    // NormalExp.h:1356-1399
GPURAND_FREE2(cauchy, GR_CAUCHY, 0, 1)          // NormalExp.h:1090-1131
GPURAND_FREE2(weibull, GR_WEIBULL, 1, 1)        // NormalExp.h:1658-1701
GPURAND_FREE2(extremeValue, GR_EXTREME_VALUE, 0, 1)  // NormalExp.h:1770-1815
GPURAND_FREE2(gamma, GR_GAMMA, 1, 1)            // NormalExp.h:1610-1651
GPURAND_FREE2(beta, GR_BETA, 1, 1)              // NormalExp.h:1043-1083
GPURAND_FREE2(fisherF, GR_FISHER_F, 1, 1)       // NormalExp.h:1929-1970

// normal(rows, cols, urng) is StdNormalGen; normal(rows, cols, urng, mean,
// stdev = 1) is NormalGen (NormalExp.h:1198-1286)
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> normal(Index rows, Index cols, Urng& urng) {
  return {rows, cols, urng, gpurand::detail::desc(GR_NORMAL_STD, gpurand::dtype_of<typename Derived::Scalar>::value)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> normal(Index rows, Index cols, Urng& urng, typename Derived::Scalar mean,
                                      typename Derived::Scalar stdev = 1) {
  return {rows, cols, urng,
          gpurand::detail::desc(GR_NORMAL, gpurand::dtype_of<typename Derived::Scalar>::value, mean, stdev)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> normalLike(const Derived& o, Urng& urng) {
  return normal<Derived>(o.rows(), o.cols(), urng);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> normalLike(const Derived& o, Urng& urng, typename Derived::Scalar mean,
                                          typename Derived::Scalar stdev = 1) {
  return normal<Derived>(o.rows(), o.cols(), urng, mean, stdev);
}
// uniformReal(rows, cols, urng, min, max) is UniformRealGen (Basic.h:1019-1062)
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> uniformReal(Index rows, Index cols, Urng& urng, typename Derived::Scalar min,
                                           typename Derived::Scalar max) {
  return {rows, cols, urng,
          gpurand::detail::desc(GR_UNIFORM_REAL2, gpurand::dtype_of<typename Derived::Scalar>::value, min, max)};
}
// balanced(rows, cols, urng, a, b) is Balanced2Gen (Basic.h:886-949)
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> balanced(Index rows, Index cols, Urng& urng, typename Derived::Scalar a,
                                        typename Derived::Scalar b) {
  return {rows, cols, urng,
          gpurand::detail::desc(GR_BALANCED2, gpurand::dtype_of<typename Derived::Scalar>::value, a, b)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> exponential(Index rows, Index cols, Urng& urng, typename Derived::Scalar lambda = 1) {
  return {rows, cols, urng,
          gpurand::detail::desc(GR_EXPONENTIAL, gpurand::dtype_of<typename Derived::Scalar>::value, lambda)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> exponentialLike(const Derived& o, Urng& urng, typename Derived::Scalar lambda = 1) {
  return exponential<Derived>(o.rows(), o.cols(), urng, lambda);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> studentT(Index rows, Index cols, Urng& urng, typename Derived::Scalar n = 1) {
  return {rows, cols, urng, gpurand::detail::desc(GR_STUDENT_T, gpurand::dtype_of<typename Derived::Scalar>::value, n)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> studentTLike(const Derived& o, Urng& urng, typename Derived::Scalar n = 1) {
  return studentT<Derived>(o.rows(), o.cols(), urng, n);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> chiSquared(Index rows, Index cols, Urng& urng, typename Derived::Scalar n = 1) {
  return {rows, cols, urng,
          gpurand::detail::desc(GR_CHI_SQUARED, gpurand::dtype_of<typename Derived::Scalar>::value, n)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> chiSquaredLike(const Derived& o, Urng& urng, typename Derived::Scalar n = 1) {
  return chiSquared<Derived>(o.rows(), o.cols(), urng, n);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> bernoulli(Index rows, Index cols, Urng& urng, double p = 0.5) {
  return {rows, cols, urng, gpurand::detail::desc(GR_BERNOULLI, gpurand::dtype_of<typename Derived::Scalar>::value, p)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> bernoulliLike(const Derived& o, Urng& urng, double p = 0.5) {
  return bernoulli<Derived>(o.rows(), o.cols(), urng, p);
}
// integer kinds (Discrete.h:1381-1900)
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> uniformInt(Index rows, Index cols, Urng& urng, typename Derived::Scalar min,
                                          typename Derived::Scalar max) {
  return {rows, cols, urng, gpurand::detail::desc(GR_UNIFORM_INT, GR_I32, min, max)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> uniformIntLike(const Derived& o, Urng& urng, typename Derived::Scalar min,
                                              typename Derived::Scalar max) {
  return uniformInt<Derived>(o.rows(), o.cols(), urng, min, max);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> poisson(Index rows, Index cols, Urng& urng, double mean = 1) {
  return {rows, cols, urng, gpurand::detail::desc(GR_POISSON, GR_I32, mean)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> poissonLike(const Derived& o, Urng& urng, double mean = 1) {
  return poisson<Derived>(o.rows(), o.cols(), urng, mean);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> binomial(Index rows, Index cols, Urng& urng, typename Derived::Scalar trials = 1,
                                        double p = 0.5) {
  return {rows, cols, urng, gpurand::detail::desc(GR_BINOMIAL, GR_I32, p, 0, trials)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> binomialLike(const Derived& o, Urng& urng, typename Derived::Scalar trials = 1,
                                            double p = 0.5) {
  return binomial<Derived>(o.rows(), o.cols(), urng, trials, p);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> negativeBinomial(Index rows, Index cols, Urng& urng, typename Derived::Scalar trials = 1,
                                                double p = 0.5) {
  return {rows, cols, urng, gpurand::detail::desc(GR_NEGATIVE_BINOMIAL, GR_I32, p, 0, trials)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> negativeBinomialLike(const Derived& o, Urng& urng, typename Derived::Scalar trials = 1,
                                                    double p = 0.5) {
  return negativeBinomial<Derived>(o.rows(), o.cols(), urng, trials, p);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> geometric(Index rows, Index cols, Urng& urng, double p = 0.5) {
  return {rows, cols, urng, gpurand::detail::desc(GR_GEOMETRIC, GR_I32, p)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> geometricLike(const Derived& o, Urng& urng, double p = 0.5) {
  return geometric<Derived>(o.rows(), o.cols(), urng, p);
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> discrete(Index rows, Index cols, Urng& urng, std::initializer_list<double> weights) {
  return {rows, cols, urng, gpurand::detail::desc(GR_DISCRETE, GR_I32), std::vector<double>(weights)};
}
template <typename Derived, typename Urng, typename It>
inline RandExpr<Derived, Urng> discrete(Index rows, Index cols, Urng& urng, It first, It last) {
  return {rows, cols, urng, gpurand::detail::desc(GR_DISCRETE, GR_I32), std::vector<double>(first, last)};
}
template <typename Derived, typename Urng>
inline RandExpr<Derived, Urng> discreteLike(const Derived& o, Urng& urng, std::initializer_list<double> weights) {
  return discrete<Derived>(o.rows(), o.cols(), urng, weights);
}
#undef GPURAND_FREE0
#undef GPURAND_FREE2

// ---- per-element parameters (the *VGen overloads) -------------------------------
// normal(urng, mean, stdev) with arrays of the output's shape (NormalVGen,
// NormalExp.h:1295-1340); a scalar operand takes the other overloads.
template <typename Scalar>
inline gpurand::DeviceArray<Scalar> normal(Vmt19937_64& urng, const gpurand::DeviceArray<Scalar>& mean,
                                           const gpurand::DeviceArray<Scalar>& stdev) {
  if (mean.rows() != stdev.rows() || mean.cols() != stdev.cols()) throw std::invalid_argument("normal: shapes differ");
  gpurand::DeviceArray<Scalar> out(mean.rows(), mean.cols());
  const gr_dist_desc d = gpurand::detail::desc(GR_NORMAL, gpurand::dtype_of<Scalar>::value);
  gpurand::check(gr_sample_v2(urng.handle(), &d, mean.data(), stdev.data(), out.data(), (size_t)out.size(),
                              urng.stream()),
                 "normal");
  return out;
}
template <typename Scalar>
inline gpurand::DeviceArray<Scalar> uniformReal(Vmt19937_64& urng, const gpurand::DeviceArray<Scalar>& a,
                                                const gpurand::DeviceArray<Scalar>& b) {
  if (a.rows() != b.rows() || a.cols() != b.cols()) throw std::invalid_argument("uniformReal: shapes differ");
  gpurand::DeviceArray<Scalar> out(a.rows(), a.cols());
  const gr_dist_desc d = gpurand::detail::desc(GR_UNIFORM_REAL2, gpurand::dtype_of<Scalar>::value);
  gpurand::check(gr_sample_v2(urng.handle(), &d, a.data(), b.data(), out.data(), (size_t)out.size(), urng.stream()),
                 "uniformReal");
  return out;
}
// binomial(urng, trials, p) (BinomialVGen<int32_t>, Discrete.h:1822-1898)
inline gpurand::DeviceArray<int32_t> binomial(Vmt19937_64& urng, const gpurand::DeviceArray<int32_t>& trials,
                                              const gpurand::DeviceArray<float>& p) {
  if (trials.rows() != p.rows() || trials.cols() != p.cols()) throw std::invalid_argument("binomial: shapes differ");
  gpurand::DeviceArray<int32_t> out(p.rows(), p.cols());
  const gr_dist_desc d = gpurand::detail::desc(GR_BINOMIAL, GR_I32);
  gpurand::check(gr_sample_v2(urng.handle(), &d, trials.data(), p.data(), out.data(), (size_t)out.size(),
                              urng.stream()),
                 "binomial");
  return out;
}

// ---- multivariate generators (MvDists/*.h) ---------------------------------------
// generate(urng, samples) returns the reference's layout: dim x samples
// (Wishart: dim x (dim * samples)).  Host matrices are column-major doubles.
template <typename _Scalar>
class MvNormalGen {
 public:
  MvNormalGen(const std::vector<double>& mean, const std::vector<double>& cov, bool lower_triangular = false)
      : dim_((int32_t)mean.size()) {
    gpurand::check(gr_mvnormal_create(&g_, gpurand::dtype_of<_Scalar>::value, dim_, mean.data(), cov.data(),
                                      lower_triangular ? GR_MATRIX_LOWER : GR_MATRIX_FULL),
                   "MvNormalGen");
  }
  MvNormalGen(const MvNormalGen&) = delete;
  MvNormalGen& operator=(const MvNormalGen&) = delete;
  ~MvNormalGen() {
    if (g_) gr_mvnormal_destroy(g_);
  }
  gpurand::DeviceArray<_Scalar> generate(Vmt19937_64& urng, Index samples) {
    gpurand::DeviceArray<_Scalar> out(dim_, samples);
    gpurand::check(gr_mvnormal_sample(g_, urng.handle(), out.data(), (size_t)samples, urng.stream()), "generate");
    return out;
  }
  Index dims() const { return dim_; }

 private:
  gr_mvnormal* g_ = nullptr;
  int32_t dim_;
};

template <typename _Scalar, int32_t INVERSE>
class WishartGenT {
 public:
  WishartGenT(int64_t df, const std::vector<double>& scale, int32_t dim, bool lower_triangular = false) : dim_(dim) {
    gpurand::check(gr_wishart_create(&g_, gpurand::dtype_of<_Scalar>::value, dim, df, scale.data(),
                                     lower_triangular ? GR_MATRIX_LOWER : GR_MATRIX_FULL, INVERSE),
                   "WishartGen");
  }
  WishartGenT(const WishartGenT&) = delete;
  WishartGenT& operator=(const WishartGenT&) = delete;
  ~WishartGenT() {
    if (g_) gr_wishart_destroy(g_);
  }
  gpurand::DeviceArray<_Scalar> generate(Vmt19937_64& urng, Index samples) {
    gpurand::DeviceArray<_Scalar> out(dim_, dim_ * samples);
    gpurand::check(gr_wishart_sample(g_, urng.handle(), out.data(), (size_t)samples, urng.stream()), "generate");
    return out;
  }
  Index dims() const { return dim_; }

 private:
  gr_wishart* g_ = nullptr;
  int32_t dim_;
};
template <typename _Scalar>
using WishartGen = WishartGenT<_Scalar, 0>;
template <typename _Scalar>
using InvWishartGen = WishartGenT<_Scalar, 1>;

template <typename _Scalar>
class DirichletGen {
 public:
  explicit DirichletGen(const std::vector<double>& alpha) : dim_((int32_t)alpha.size()) {
    gpurand::check(gr_dirichlet_create(&g_, gpurand::dtype_of<_Scalar>::value, dim_, alpha.data()), "DirichletGen");
  }
  DirichletGen(const DirichletGen&) = delete;
  DirichletGen& operator=(const DirichletGen&) = delete;
  ~DirichletGen() {
    if (g_) gr_dirichlet_destroy(g_);
  }
  gpurand::DeviceArray<_Scalar> generate(Vmt19937_64& urng, Index samples) {
    gpurand::DeviceArray<_Scalar> out(dim_, samples);
    gpurand::check(gr_dirichlet_sample(g_, urng.handle(), out.data(), (size_t)samples, urng.stream()), "generate");
    return out;
  }
  Index dims() const { return dim_; }

 private:
  gr_dirichlet* g_ = nullptr;
  int32_t dim_;
};

template <typename _Scalar = int32_t>
class MultinomialGen {
  static_assert(std::is_same<_Scalar, int32_t>::value, "MultinomialGen: int32_t only");

 public:
  MultinomialGen(int32_t trials, const std::vector<double>& probs) : dim_((int32_t)probs.size()) {
    gpurand::check(gr_multinomial_create(&g_, dim_, trials, probs.data()), "MultinomialGen");
  }
  MultinomialGen(const MultinomialGen&) = delete;
  MultinomialGen& operator=(const MultinomialGen&) = delete;
  ~MultinomialGen() {
    if (g_) gr_multinomial_destroy(g_);
  }
  gpurand::DeviceArray<int32_t> generate(Vmt19937_64& urng, Index samples) {
    gpurand::DeviceArray<int32_t> out(dim_, samples);
    gpurand::check(gr_multinomial_sample(g_, urng.handle(), out.data(), (size_t)samples, urng.stream()), "generate");
    return out;
  }
  Index dims() const { return dim_; }

 private:
  gr_multinomial* g_ = nullptr;
  int32_t dim_;
};

// makeMvNormalGen / makeWishartGen / makeDirichletGen / makeMultinomialGen
// (MvNormal.h:130-170, Multinomial.h:125-158)
template <typename _Scalar>
inline MvNormalGen<_Scalar> makeMvNormalGen(const std::vector<double>& mean, const std::vector<double>& cov) {
  return MvNormalGen<_Scalar>(mean, cov);
}

}  // namespace Rand
}  // namespace Eigen

#endif
