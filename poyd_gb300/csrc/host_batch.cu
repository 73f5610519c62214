// Host-buffer batched align_2 with the download overlapping the DP.
//
// A caller whose sequences live in host memory (an OCaml stub holding seq
// blocks) would otherwise upload the batch, run poyd_align_2_batch and then
// download every result: the download adds to the DP time.  Here the batch
// is uploaded and run as one DP launch whose output slots are laid out in
// the DP's own longest-first order.  The fused traceback raises a flag in
// host-mapped memory as each batch of 32 pairs is written, so the finished
// slots form a growing prefix of the output.  The host follows that prefix
// and copies it down on a second stream while the DP runs; only the slots
// of the last (shortest) pairs are copied after it.  Cutting the batch into
// separate launches was measured slower: each launch gives up part of the
// longest-first schedule's load balance.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "poyd_internal.h"

namespace poyd {

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

int ensure(DevBuf &b, size_t need) {
  if (need <= b.cap) return POYD_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  need = std::max<size_t>(need, 256);
  if (cudaMalloc(&b.p, need) != cudaSuccess) {
    cudaGetLastError();
    return fail(POYD_ENOMEM, "host batch: device allocation of %zu bytes failed", need);
  }
  b.cap = need;
  return POYD_OK;
}

struct Pipe {
  std::mutex mu;
  bool ready = false;
  cudaStream_t dp = nullptr, copy = nullptr;
  DevBuf seq, off, len, out, olen, cost;
  int *flags_h = nullptr;  // host-mapped batch flags
  int *flags_d = nullptr;
  size_t flags_cap = 0;
};

Pipe &pipe_for(int dev) {
  static Pipe pipes[64];
  return pipes[dev & 63];
}

// POYD_PIPE_TRACE=1 prints, per download issued, the host time and the
// bytes, and the host times of upload, launch and completion (stderr).
struct Trace {
  bool on = std::getenv("POYD_PIPE_TRACE") != nullptr;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
        .count();
  }
  void log(const char *what, long long a = 0, long long b = 0) const {
    if (on) std::fprintf(stderr, "%9.3f ms  %s %lld %lld\n", ms(), what, a, b);
  }
};

// Waits for both streams when the call returns, whichever way: an early
// error return must not leave a download still writing into the caller's
// buffers, or the DP still writing into the pipe's buffers.
struct Drain {
  Pipe &P;
  ~Drain() {
    if (!P.ready) return;
    cudaStreamSynchronize(P.dp);
    cudaStreamSynchronize(P.copy);
  }
};

#define CKH(call)                                        \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

}  // namespace

}  // namespace poyd

using namespace poyd;

extern "C" int poyd_align_2_host(const poyd_cm *cm, int32_t n, const uint8_t *seq,
                                 const int64_t *a_off, const int32_t *a_len,
                                 const int64_t *b_off, const int32_t *b_len, int32_t *cost,
                                 uint8_t *out, int64_t out_cap, int64_t *out_off,
                                 int32_t *out_len, int32_t flags) {
  if (!cm) return fail(POYD_EINVAL, "poyd_align_2_host: null cost matrix");
  if (n < 0 || (n > 0 && (!seq || !a_off || !a_len || !b_off || !b_len || !cost || !out ||
                          !out_off || !out_len)))
    return fail(POYD_EINVAL, "poyd_align_2_host: null argument");
  if (n == 0) return POYD_OK;
  Trace T;
  int dev = 0;
  CKH(cudaGetDevice(&dev));
  Pipe &P = pipe_for(dev);
  std::lock_guard<std::mutex> guard(P.mu);
  if (!P.ready) {
    CKH(cudaStreamCreateWithFlags(&P.dp, cudaStreamNonBlocking));
    CKH(cudaStreamCreateWithFlags(&P.copy, cudaStreamNonBlocking));
    P.ready = true;
  }
  Drain drain{P};
  int64_t lo = INT64_MAX, hi = 0, slots = 0;
  for (int32_t i = 0; i < n; ++i) {
    if (a_len[i] < 1 || b_len[i] < 1)
      return fail(POYD_EINVAL, "sequences must have length >= 1 (the leading gap)");
    lo = std::min({lo, a_off[i], b_off[i]});
    hi = std::max({hi, a_off[i] + a_len[i], b_off[i] + b_len[i]});
    slots += 4 * slot_cap(a_len[i], b_len[i]);
  }
  if (slots > out_cap)
    return fail(POYD_ERANGE, "output slots need %lld bytes, capacity %lld", (long long)slots,
                (long long)out_cap);
  const size_t nb = ((size_t)n + kLanes - 1) / kLanes;
  int rc = ensure(P.seq, (size_t)(hi - lo) + 64);
  if (!rc) rc = ensure(P.off, sizeof(int64_t) * 3 * (size_t)n);
  if (!rc) rc = ensure(P.len, sizeof(int32_t) * 2 * (size_t)n);
  if (!rc) rc = ensure(P.out, (size_t)slots);
  if (!rc) rc = ensure(P.olen, sizeof(int32_t) * 2 * (size_t)n);
  if (!rc) rc = ensure(P.cost, sizeof(int32_t) * (size_t)n);
  if (rc) return rc;
  if (nb > P.flags_cap) {
    if (P.flags_h) cudaFreeHost(P.flags_h);
    P.flags_h = nullptr;
    P.flags_cap = 0;
    CKH(cudaHostAlloc((void **)&P.flags_h, sizeof(int) * nb, cudaHostAllocMapped));
    CKH(cudaHostGetDevicePointer((void **)&P.flags_d, P.flags_h, 0));
    P.flags_cap = nb;
  }
  std::memset(P.flags_h, 0, sizeof(int) * nb);

  // upload: the sequences' byte range and the pairs' offsets (rebased) and
  // lengths
  std::vector<int64_t> off(2 * (size_t)n);
  std::vector<int32_t> len(2 * (size_t)n);
  for (int32_t i = 0; i < n; ++i) {
    off[i] = a_off[i] - lo;
    off[n + i] = b_off[i] - lo;
    len[i] = a_len[i];
    len[n + i] = b_len[i];
  }
  int64_t *off_d = (int64_t *)P.off.p;
  int32_t *len_d = (int32_t *)P.len.p;
  T.log("upload", hi - lo);
  CKH(cudaMemcpyAsync(P.seq.p, seq + lo, (size_t)(hi - lo), cudaMemcpyHostToDevice, P.dp));
  CKH(cudaMemcpyAsync(off_d, off.data(), sizeof(int64_t) * 2 * (size_t)n, cudaMemcpyHostToDevice,
                      P.dp));
  CKH(cudaMemcpyAsync(len_d, len.data(), sizeof(int32_t) * 2 * (size_t)n, cudaMemcpyHostToDevice,
                      P.dp));
  uint8_t *out_d = (uint8_t *)P.out.p;
  int32_t *olen_d = (int32_t *)P.olen.p, *cost_d = (int32_t *)P.cost.p;
  LinStream ls;
  ls.a_len_h = a_len;
  ls.b_len_h = b_len;
  ls.out_off_host = out_off;
  ls.out_off_dev = off_d + 2 * (size_t)n;
  ls.done = P.flags_d;
  bool streamed = cm->cost_model != 1;
  if (streamed) {
    rc = align_2_streamed(cm, n, (const uint8_t *)P.seq.p, off_d, len_d, off_d + n, len_d + n,
                          cost_d, out_d, olen_d, flags, &ls, P.dp);
    streamed = !rc && ls.waves == 1;
  } else {
    // affine: slots in pair order, downloaded after the DP
    int64_t o = 0;
    for (int32_t i = 0; i < n; ++i) {
      out_off[i] = o;
      o += 4 * slot_cap(a_len[i], b_len[i]);
    }
    CKH(cudaMemcpyAsync(off_d + 2 * (size_t)n, out_off, sizeof(int64_t) * (size_t)n,
                        cudaMemcpyHostToDevice, P.dp));
    rc = poyd_align_2_batch(cm, n, (const uint8_t *)P.seq.p, off_d, len_d, off_d + n, len_d + n,
                            cost_d, out_d, off_d + 2 * (size_t)n, olen_d, nullptr, flags, P.dp);
  }
  if (rc) return rc;
  T.log("launched", streamed);
  int64_t sent = 0;
  if (streamed) {
    // bytes of the slots of order positions < p
    std::vector<int64_t> prefix((size_t)n + 1, 0);
    for (int32_t p = 0; p < n; ++p)
      prefix[p + 1] = prefix[p] + 4 * slot_cap(a_len[ls.order[p]], b_len[ls.order[p]]);
    const int64_t step = std::max<int64_t>(slots / 32, 1 << 20);
    volatile int *fl = P.flags_h;
    size_t q = 0;  // batches [0, q) are finished
    for (;;) {
      while (q < nb && fl[q]) ++q;
      const int64_t ready = prefix[std::min((size_t)n, q * kLanes)];
      if (q == nb) break;
      if (ready - sent >= step) {
        CKH(cudaMemcpyAsync(out + sent, out_d + sent, (size_t)(ready - sent),
                            cudaMemcpyDeviceToHost, P.copy));
        T.log("download", sent, ready - sent);
        sent = ready;
      }
      const cudaError_t e = cudaStreamQuery(P.dp);
      if (e != cudaErrorNotReady) {  // finished (or failed): no more flags will come
        if (e != cudaSuccess) return cuda_fail(e, "poyd_align_2_host");
        break;
      }
      std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
  }
  CKH(cudaStreamSynchronize(P.dp));
  T.log("dp done", sent);
  if (slots > sent)
    CKH(cudaMemcpyAsync(out + sent, out_d + sent, (size_t)(slots - sent), cudaMemcpyDeviceToHost,
                        P.copy));
  CKH(cudaMemcpyAsync(cost, cost_d, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, P.copy));
  CKH(cudaMemcpyAsync(out_len, olen_d, sizeof(int32_t) * 2 * (size_t)n, cudaMemcpyDeviceToHost,
                      P.copy));
  CKH(cudaStreamSynchronize(P.copy));
  T.log("done", slots - sent);
  for (int32_t i = 0; i < n; ++i)
    if (out_len[2 * (size_t)i] < 0 || out_len[2 * (size_t)i + 1] < 0)
      return fail(POYD_ECUDA, "traceback failed for pair %d", i);
  return POYD_OK;
}
