// Internal declarations shared by the host (.cpp) and device (.cu) halves of
// libtc.  Nothing here is part of the C ABI.
#pragma once
#include <stdint.h>
#include <stdarg.h>
#include <string>
#include "../../include/tc.h"

namespace tc {

// Error text of calls made without a ctx (thread-local).
void set_global_error(const char *fmt, ...);
const char *global_error();

// Chung-Lu cumulative weight table (host); the device generator uploads the
// same table, so host and device samples agree bit for bit.
void chung_lu_table(int64_t n, double avg_degree, double gamma, uint64_t *cum);

// R-MAT integer thresholds t1 < t2 < t3 from (a, b, c).
void rmat_thresholds(double a, double b, double c, uint64_t *t1, uint64_t *t2, uint64_t *t3);

// Bits needed to hold values in [0, x] (at least 1).
static inline int bit_width_u64(uint64_t x) {
  int b = 1;
  while (b < 64 && (x >> b) != 0) ++b;
  return b;
}

}  // namespace tc
