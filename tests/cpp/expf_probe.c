/* Test probe: the product's exponential (kdgr_math.h, the function the
 * plain kernel calls) compiled for the host, so a test can compare it with
 * the oracle's own restatement of the same method. */
#include <stdint.h>

#include "kdgr_math.h"

void probe_expf_n(const float* x, float* y, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) y[i] = kdgr_expf(x[i]);
}
