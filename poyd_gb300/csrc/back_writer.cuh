// Backward byte writer shared by the traceback kernels.
#pragma once
#include <cstdint>

namespace poyd {

// Writes a sequence backwards (the reference's seq_prepend order), collecting
// bytes in a register and storing whole aligned 4-byte words; only a word
// that the sequence covers in part (its two ends) is written byte by byte.
struct BackWriter {
  uint8_t *p;     // next position (moves down)
  uint32_t buf;   // pending bytes; the last one written in the low byte
  int pend;
  __device__ explicit BackWriter(uint8_t *top) : p(top), buf(0), pend(0) {}
  __device__ __forceinline__ void put(uint32_t v) {
    buf = (buf << 8) | v;
    ++pend;
    if (((uintptr_t)p & 3u) == 0) {  // p is the lowest byte of its word
      if (pend == 4) *(uint32_t *)p = buf;
      else
        for (int i = 0; i < pend; ++i) p[i] = (uint8_t)(buf >> (8 * i));
      pend = 0;
    }
    --p;
  }
  __device__ __forceinline__ void flush() {  // bytes at p+1 .. p+pend
    for (int i = 0; i < pend; ++i) p[1 + i] = (uint8_t)(buf >> (8 * i));
    pend = 0;
  }
};

}  // namespace poyd
