// Affine-gap ("3 matrix") DO path (affine.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "poyd_internal.h"

namespace poyd {

// Batched algn_CAML_cost_affine_3 (want_align = false) or
// algn_CAML_align_affine_3 (want_align = true) over caller-order pairs.
int affine_batch(const poyd_cm *cm, int maxc, int32_t n, const uint8_t *seq,
                 const int64_t *a_off, const int32_t *a_len, const int64_t *b_off,
                 const int32_t *b_len, int32_t *cost, int64_t *cells, bool want_align,
                 int32_t flags, uint8_t *out, const int64_t *out_off, int32_t *out_len,
                 cudaStream_t st);

}  // namespace poyd
