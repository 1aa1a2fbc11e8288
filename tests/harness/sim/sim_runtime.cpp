// Host stand-ins for the CUDA runtime calls that libgbcc's host code makes
// (see sim.hpp).  One simulated device with 152 SMs.  Device and pinned
// memory are host memory.  Work on a stream runs at once unless the stream is
// being captured; then it is recorded, and cudaGraphLaunch runs the record.
// As under CUDA:
//   - memory that cudaMallocAsync returns during a capture belongs to the
//     graph and keeps its address at every launch;
//   - synchronising calls made from the capturing thread fail
//     (cudaStreamSynchronize of the capturing stream, cudaMemcpy, cudaMemset,
//     cudaMalloc), and so do copies between a capturing stream and pageable
//     host memory.
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "sim.hpp"

namespace {

struct Stream {
  bool capturing = false;
  std::vector<sim::Op> ops;
  std::vector<void *> mem;  // allocated during the capture
};

struct Graph {
  std::vector<sim::Op> ops;
  std::vector<void *> mem;
};

Stream g_default;
thread_local int t_captures = 0;  // streams this thread is capturing
std::mutex g_mu;
std::map<const char *, size_t> g_pinned;  // page-locked ranges: base -> bytes

Stream *S(cudaStream_t s) { return s ? reinterpret_cast<Stream *>(s) : &g_default; }

void *alloc_bytes(size_t n) {
  const size_t a = 256;
  return std::aligned_alloc(a, ((n ? n : 1) + a - 1) / a * a);
}

bool pinned(const void *p, size_t n) {
  std::lock_guard<std::mutex> lk(g_mu);
  const char *c = static_cast<const char *>(p);
  auto it = g_pinned.upper_bound(c);
  if (it == g_pinned.begin()) return false;
  --it;
  return c >= it->first && c + n <= it->first + it->second;
}

}  // namespace

namespace sim {

void submit(cudaStream_t s, Op op) {
  Stream *st = S(s);
  if (st->capturing) st->ops.push_back(std::move(op));
  else op();
}

bool capturing(cudaStream_t s) { return S(s)->capturing; }

}  // namespace sim

extern "C" {

cudaError_t cudaGetDeviceCount(int *n) {
  *n = 1;
  return cudaSuccess;
}
cudaError_t cudaSetDevice(int d) { return d == 0 ? cudaSuccess : cudaErrorInvalidDevice; }
cudaError_t cudaGetDevice(int *d) {
  *d = 0;
  return cudaSuccess;
}
cudaError_t cudaDeviceGetAttribute(int *v, enum cudaDeviceAttr attr, int) {
  *v = attr == cudaDevAttrMultiProcessorCount ? 152 : 0;
  return cudaSuccess;
}
cudaError_t cudaDeviceGetDefaultMemPool(cudaMemPool_t *pool, int) {
  *pool = nullptr;
  return cudaSuccess;
}
cudaError_t cudaMemPoolSetAttribute(cudaMemPool_t, enum cudaMemPoolAttr, void *) {
  return cudaSuccess;
}
cudaError_t cudaMemPoolGetAttribute(cudaMemPool_t, enum cudaMemPoolAttr, void *v) {
  *static_cast<unsigned long long *>(v) = 0;
  return cudaSuccess;
}
cudaError_t cudaMemGetInfo(size_t *free_b, size_t *total) {
  *total = (size_t)280 << 30;
  *free_b = (size_t)270 << 30;
  return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) {
  return t_captures ? cudaErrorStreamCaptureUnsupported : cudaSuccess;
}
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
cudaError_t cudaPeekAtLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t e) {
  switch (e) {
    case cudaSuccess: return "no error";
    case cudaErrorStreamCaptureUnsupported: return "operation not permitted when stream is capturing";
    case cudaErrorStreamCaptureImplicit: return "operation would make the legacy stream depend on a capturing blocking stream";
    case cudaErrorInvalidValue: return "invalid argument";
    default: return "simulated CUDA error";
  }
}

cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned int) {
  *s = reinterpret_cast<cudaStream_t>(new Stream());
  return cudaSuccess;
}
cudaError_t cudaStreamCreate(cudaStream_t *s) { return cudaStreamCreateWithFlags(s, 0); }
cudaError_t cudaStreamDestroy(cudaStream_t s) {
  if (s) delete reinterpret_cast<Stream *>(s);
  return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t s) {
  return S(s)->capturing ? cudaErrorStreamCaptureUnsupported : cudaSuccess;
}
cudaError_t cudaStreamIsCapturing(cudaStream_t s, enum cudaStreamCaptureStatus *st) {
  *st = S(s)->capturing ? cudaStreamCaptureStatusActive : cudaStreamCaptureStatusNone;
  return cudaSuccess;
}
cudaError_t cudaStreamBeginCapture(cudaStream_t s, enum cudaStreamCaptureMode) {
  Stream *st = S(s);
  if (st->capturing) return cudaErrorIllegalState;
  st->capturing = true;
  st->ops.clear();
  st->mem.clear();
  ++t_captures;
  return cudaSuccess;
}
cudaError_t cudaStreamEndCapture(cudaStream_t s, cudaGraph_t *g) {
  Stream *st = S(s);
  if (!st->capturing) return cudaErrorIllegalState;
  st->capturing = false;
  --t_captures;
  auto *gr = new Graph();
  gr->ops.swap(st->ops);
  gr->mem.swap(st->mem);
  *g = reinterpret_cast<cudaGraph_t>(gr);
  return cudaSuccess;
}
cudaError_t cudaGraphInstantiate(cudaGraphExec_t *e, cudaGraph_t g, unsigned long long) {
  // the executable graph takes the recorded work and the graph's memory
  auto *gr = reinterpret_cast<Graph *>(g);
  auto *ex = new Graph();
  ex->ops = gr->ops;
  ex->mem.swap(gr->mem);
  *e = reinterpret_cast<cudaGraphExec_t>(ex);
  return cudaSuccess;
}
cudaError_t cudaGraphDestroy(cudaGraph_t g) {
  auto *gr = reinterpret_cast<Graph *>(g);
  for (void *p : gr->mem) std::free(p);
  delete gr;
  return cudaSuccess;
}
cudaError_t cudaGraphExecDestroy(cudaGraphExec_t e) {
  auto *ex = reinterpret_cast<Graph *>(e);
  for (void *p : ex->mem) std::free(p);
  delete ex;
  return cudaSuccess;
}
cudaError_t cudaGraphLaunch(cudaGraphExec_t e, cudaStream_t s) {
  auto *ex = reinterpret_cast<Graph *>(e);
  sim::submit(s, [ex]() {
    for (auto &op : ex->ops) op();
  });
  return cudaSuccess;
}

cudaError_t cudaMalloc(void **p, size_t n) {
  if (t_captures) return cudaErrorStreamCaptureUnsupported;
  *p = alloc_bytes(n);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void *p) {
  if (t_captures) return cudaErrorStreamCaptureUnsupported;
  std::free(p);
  return cudaSuccess;
}
cudaError_t cudaMallocAsync(void **p, size_t n, cudaStream_t s) {
  *p = alloc_bytes(n);
  if (!*p) return cudaErrorMemoryAllocation;
  if (S(s)->capturing) S(s)->mem.push_back(*p);
  return cudaSuccess;
}
cudaError_t cudaFreeAsync(void *p, cudaStream_t s) {
  Stream *st = S(s);
  if (st->capturing) {
    for (void *q : st->mem)
      if (q == p) return cudaSuccess;  // graph memory: freed with the graph
    return cudaErrorInvalidValue;      // not modelled: freeing outside memory in a capture
  }
  std::free(p);
  return cudaSuccess;
}
cudaError_t cudaHostAlloc(void **p, size_t n, unsigned int) {
  *p = alloc_bytes(n);
  if (!*p) return cudaErrorMemoryAllocation;
  std::lock_guard<std::mutex> lk(g_mu);
  g_pinned[static_cast<const char *>(*p)] = n;
  return cudaSuccess;
}
cudaError_t cudaMallocHost(void **p, size_t n) { return cudaHostAlloc(p, n, 0); }
cudaError_t cudaFreeHost(void *p) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_pinned.erase(static_cast<const char *>(p));
  }
  std::free(p);
  return cudaSuccess;
}

cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, enum cudaMemcpyKind) {
  if (t_captures) return cudaErrorStreamCaptureImplicit;
  std::memmove(dst, src, n);
  return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void *dst, const void *src, size_t n, enum cudaMemcpyKind kind,
                            cudaStream_t s) {
  if (S(s)->capturing) {
    const bool host_src = kind == cudaMemcpyHostToDevice || kind == cudaMemcpyHostToHost;
    const bool host_dst = kind == cudaMemcpyDeviceToHost || kind == cudaMemcpyHostToHost;
    if ((host_src && !pinned(src, n)) || (host_dst && !pinned(dst, n)))
      return cudaErrorStreamCaptureUnsupported;
  }
  sim::submit(s, [dst, src, n]() { std::memmove(dst, src, n); });
  return cudaSuccess;
}
cudaError_t cudaMemset(void *p, int v, size_t n) {
  if (t_captures) return cudaErrorStreamCaptureImplicit;
  std::memset(p, v, n);
  return cudaSuccess;
}
cudaError_t cudaMemsetAsync(void *p, int v, size_t n, cudaStream_t s) {
  sim::submit(s, [p, v, n]() { std::memset(p, v, n); });
  return cudaSuccess;
}

struct SimEvent {
  int unused = 0;
};
cudaError_t cudaEventCreate(cudaEvent_t *e) {
  *e = reinterpret_cast<cudaEvent_t>(new SimEvent());
  return cudaSuccess;
}
cudaError_t cudaEventCreateWithFlags(cudaEvent_t *e, unsigned int) { return cudaEventCreate(e); }
cudaError_t cudaEventDestroy(cudaEvent_t e) {
  delete reinterpret_cast<SimEvent *>(e);
  return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0.0f;
  return cudaSuccess;
}

}  // extern "C"
