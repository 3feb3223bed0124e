// Host build of the library's integer-arithmetic double log / exp
// (eigenrand_gb300/csrc/gr_dmath.h) for the accuracy tests.
#include <stddef.h>

#include "gr_dmath.h"

extern "C" void grd_log_n(const double* x, double* y, size_t n) {
  for (size_t i = 0; i < n; ++i) y[i] = gr::grd_log(x[i]);
}
extern "C" void grd_exp_n(const double* x, double* y, size_t n) {
  for (size_t i = 0; i < n; ++i) y[i] = gr::grd_exp(x[i]);
}
