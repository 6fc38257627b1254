// Transfers between pageable host memory and the device through pinned bounce
// chunks that the library owns.
//
// A cudaMemcpyAsync from or to pageable memory lets the driver reach the
// caller's pages itself.  On the Grace host of a GB300 that runs at 150-180
// GB/s once the pages' translations are warm (0.8 ms for the 132 MB of
// inputs of a 128^3 solve), but the first transfer from a buffer the device
// has not touched for a second or two, or into freshly mapped pages, took 5 to
// 47 ms for the same 100-130 MB.  Here host threads copy the caller's pages
// into a small ring of pinned chunks while the copy engine moves the chunks
// filled before them; the device only ever touches the ring, which every
// transfer reuses, and the host threads' own page walks are cheap.
//
// Each worker thread owns kDepth chunk slots and handles chunks w, w+W, ...
// of the transfer; a slot is refilled only after the event recorded behind
// its previous copy has completed, so the ring can be shared by plans on
// different streams (transfers take the ring's lock one at a time).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "plan.h"

namespace marie {

namespace {

constexpr size_t kChunk = 4u << 20;      // bytes per bounce chunk
constexpr int kDepth = 2;                // chunks in flight per worker
constexpr size_t kMinBounce = 8u << 20;  // smaller pageable transfers go direct

struct Ring {
  int workers = 0;
  char* buf = nullptr;          // workers * kDepth * kChunk pinned bytes
  std::vector<cudaEvent_t> ev;  // one per slot, recorded behind the slot's last copy
  std::mutex mu;                // one transfer at a time
  bool ok = false;
};

std::mutex g_rings_mu;
std::map<int, Ring*> g_rings;  // device -> ring; kept for the life of the process

int worker_count() {
  const unsigned hc = std::thread::hardware_concurrency();
  if (hc >= 16) return 8;
  if (hc >= 4) return (int)hc / 2;
  return 1;
}

// The device's ring, created on first use; nullptr when pinned memory or
// events cannot be had (the caller then copies directly).
Ring* ring_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  std::lock_guard<std::mutex> g(g_rings_mu);
  auto it = g_rings.find(dev);
  if (it != g_rings.end()) return it->second->ok ? it->second : nullptr;
  Ring* r = new Ring;
  g_rings[dev] = r;
  r->workers = worker_count();
  const int slots = r->workers * kDepth;
  if (cudaHostAlloc(reinterpret_cast<void**>(&r->buf), (size_t)slots * kChunk, cudaHostAllocPortable) !=
      cudaSuccess) {
    cudaGetLastError();
    r->buf = nullptr;
    return nullptr;
  }
  r->ev.assign(slots, nullptr);
  for (auto& e : r->ev) {
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
  }
  r->ok = true;
  return r;
}

// Moves `bytes` between host memory and device memory on stream st.  For
// to_device the call returns once every chunk has been read from the host
// and its copy queued on st; otherwise once the host buffer holds the data.
int bounce(Ring* r, char* host, char* dev, size_t bytes, bool to_device, cudaStream_t st) {
  const size_t nch = (bytes + kChunk - 1) / kChunk;
  const int W = (int)std::min<size_t>((size_t)r->workers, nch);
  std::atomic<int> first_err{0};
  auto work = [&](int w) {
    char* slot[kDepth];
    cudaEvent_t ev[kDepth];
    for (int d = 0; d < kDepth; ++d) {
      slot[d] = r->buf + ((size_t)w * kDepth + d) * kChunk;
      ev[d] = r->ev[(size_t)w * kDepth + d];
    }
    std::vector<size_t> mine;
    for (size_t c = (size_t)w; c < nch; c += (size_t)W) mine.push_back(c);
    auto off_of = [&](size_t i) { return mine[i] * kChunk; };
    auto len_of = [&](size_t i) { return std::min(kChunk, bytes - off_of(i)); };
    auto fail = [&](cudaError_t e) {
      int z = 0;
      first_err.compare_exchange_strong(z, (int)e);
    };
    // queue the device-to-host copy of this worker's i-th chunk into its slot
    auto issue_d2h = [&](size_t i) {
      const int d = (int)(i % kDepth);
      cudaError_t e = cudaEventSynchronize(ev[d]);
      if (e == cudaSuccess) e = cudaMemcpyAsync(slot[d], dev + off_of(i), len_of(i), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaEventRecord(ev[d], st);
      return e;
    };
    if (to_device) {
      for (size_t i = 0; i < mine.size(); ++i) {
        if (first_err.load(std::memory_order_relaxed)) return;
        const int d = (int)(i % kDepth);
        cudaError_t e = cudaEventSynchronize(ev[d]);  // the slot's previous copy has finished
        if (e == cudaSuccess) {
          std::memcpy(slot[d], host + off_of(i), len_of(i));
          e = cudaMemcpyAsync(dev + off_of(i), slot[d], len_of(i), cudaMemcpyHostToDevice, st);
        }
        if (e == cudaSuccess) e = cudaEventRecord(ev[d], st);
        if (e != cudaSuccess) return fail(e);
      }
    } else {
      for (size_t i = 0; i < mine.size() && i < (size_t)kDepth; ++i) {
        const cudaError_t e = issue_d2h(i);
        if (e != cudaSuccess) return fail(e);
      }
      for (size_t i = 0; i < mine.size(); ++i) {
        if (first_err.load(std::memory_order_relaxed)) return;
        const int d = (int)(i % kDepth);
        cudaError_t e = cudaEventSynchronize(ev[d]);
        if (e == cudaSuccess) {
          std::memcpy(host + off_of(i), slot[d], len_of(i));
          if (i + kDepth < mine.size()) e = issue_d2h(i + kDepth);
        }
        if (e != cudaSuccess) return fail(e);
      }
    }
  };
  std::vector<std::thread> helpers;
  helpers.reserve(W > 1 ? W - 1 : 0);
  for (int w = 1; w < W; ++w) helpers.emplace_back(work, w);
  work(0);
  for (auto& t : helpers) t.join();
  if (const int e = first_err.load()) {
    cudaGetLastError();
    return set_error(MARIE_ECUDA, "%s transfer of %zu bytes through the pinned ring failed: %s",
                     to_device ? "host-to-device" : "device-to-host", bytes, cudaGetErrorString((cudaError_t)e));
  }
  return MARIE_OK;
}

}  // namespace

HostKind host_kind(const void* ptr) {
  cudaPointerAttributes a;
  if (!ptr || cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return HostKind::Pageable;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return HostKind::Device;
  if (a.type == cudaMemoryTypeHost) return HostKind::Pinned;
  return HostKind::Pageable;
}

int copy_to_device(void* dev, const void* host, size_t bytes, cudaStream_t st) {
  if (bytes >= kMinBounce && host_kind(host) == HostKind::Pageable) {
    if (Ring* r = ring_for_current_device()) {
      std::lock_guard<std::mutex> g(r->mu);
      return bounce(r, static_cast<char*>(const_cast<void*>(host)), static_cast<char*>(dev), bytes, true, st);
    }
  }
  MARIE_CUDA_TRY(cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, st));
  return MARIE_OK;
}

int copy_to_host(void* host, const void* dev, size_t bytes, cudaStream_t st) {
  if (bytes >= kMinBounce && host_kind(host) == HostKind::Pageable) {
    if (Ring* r = ring_for_current_device()) {
      // the data is produced by work already queued on st: wait for it before
      // taking the ring, so that other plans' transfers are not held up
      MARIE_CUDA_TRY(cudaStreamSynchronize(st));
      std::lock_guard<std::mutex> g(r->mu);
      return bounce(r, static_cast<char*>(host), static_cast<char*>(const_cast<void*>(dev)), bytes, false, st);
    }
  }
  MARIE_CUDA_TRY(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

}  // namespace marie
