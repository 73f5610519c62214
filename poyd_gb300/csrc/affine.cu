// Affine-gap DO path (placeholder until the affine kernels land).
#include "affine_kernels.cuh"

namespace poyd {

int affine_batch(const poyd_cm *, int, int32_t, const uint8_t *, const int64_t *,
                 const int32_t *, const int64_t *, const int32_t *, int32_t *, int64_t *, bool,
                 int32_t, uint8_t *, const int64_t *, int32_t *, cudaStream_t) {
  return fail(POYD_EUNSUP, "affine cost model not implemented on the GPU path yet");
}

}  // namespace poyd
