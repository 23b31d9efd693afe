// scan.cuh -- exclusive prefix sums on the device (three-phase block scan).
#pragma once

#include "common.cuh"

namespace qd {

// out[i] = sum_{j < i} in[i]; in and out may alias.  n >= 1.
void exclusive_scan_i64(Ctx* ctx, const int64_t* in, int64_t* out, int64_t n);

}  // namespace qd
