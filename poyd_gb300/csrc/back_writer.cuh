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

// Three sequences written backwards in step (one byte each per column) whose
// write positions are congruent modulo 4 (their slots are a multiple of 4
// bytes apart): one alignment check serves all three.
struct BackWriter3 {
  uint8_t *p0, *p1, *p2;
  uint32_t b0, b1, b2;
  int pend;
  __device__ BackWriter3(uint8_t *t0, uint8_t *t1, uint8_t *t2)
      : p0(t0), p1(t1), p2(t2), b0(0), b1(0), b2(0), pend(0) {}
  __device__ __forceinline__ void put(uint32_t v0, uint32_t v1, uint32_t v2) {
    b0 = (b0 << 8) | v0;
    b1 = (b1 << 8) | v1;
    b2 = (b2 << 8) | v2;
    ++pend;
    if (((uintptr_t)p0 & 3u) == 0) {
      if (pend == 4) {
        *(uint32_t *)p0 = b0;
        *(uint32_t *)p1 = b1;
        *(uint32_t *)p2 = b2;
      } else {
        for (int i = 0; i < pend; ++i) {
          p0[i] = (uint8_t)(b0 >> (8 * i));
          p1[i] = (uint8_t)(b1 >> (8 * i));
          p2[i] = (uint8_t)(b2 >> (8 * i));
        }
      }
      pend = 0;
    }
    --p0;
    --p1;
    --p2;
  }
  __device__ __forceinline__ void flush() {
    for (int i = 0; i < pend; ++i) {
      p0[1 + i] = (uint8_t)(b0 >> (8 * i));
      p1[1 + i] = (uint8_t)(b1 >> (8 * i));
      p2[1 + i] = (uint8_t)(b2 >> (8 * i));
    }
    pend = 0;
  }
};

}  // namespace poyd
