// Allocation-free scheduling entry point.
//
// Some callers cannot allocate device memory while they run: a renderer that
// owns a fixed device budget carved out at start-up (cudaMalloc could fail or
// push it over its share), or a host runtime whose GPU memory is handed out by
// its own pool (a cudaMalloc behind its back breaks its accounting, and
// cudaFree synchronises the whole device).  spray_gpu_schedule_static lets
// such callers run the speculative scheduler -- slab test of every ray against
// every domain box, (t, id)-sorted domain lists, stable partition into
// per-domain queues -- with no allocation: the scheduler's scratch lives in
// one file-scope device array of fixed size, and the caller passes only inputs
// and outputs.
//
// Limits and sharing:
//  * at most kStaticMaxRays rays, kStaticMaxDomains domains and
//    kStaticMaxEntries queue entries per call; larger requests are rejected
//    with SPRAY_GPU_EINVAL before any GPU work;
//  * the array (about 13 MB) stays allocated on every device that used this
//    library until the process exits;
//  * every call uses the same array and leaves its contents behind; the
//    counters that must start at zero are cleared by each call, so calls that
//    overlap on the GPU (different streams, or different host threads on one
//    device) race and corrupt each other -- serialise them;
//  * the call reads its entry count back and synchronises the caller's
//    stream before it returns, so it must not be made while that stream (or
//    the device) is being captured into a CUDA graph;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and keeps it for the
//    life of the process; after a cudaDeviceReset the kept address is stale,
//    so do not call this entry point again in a process that reset a device
//    it used.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/spray_gpu.h"
#include "kernels.cuh"
#include "spray_math.cuh"

namespace spray {

int fail(int code, const std::string& msg);

namespace {

constexpr int kStaticMaxRays = 1 << 18;
constexpr int kStaticMaxDomains = 256;
constexpr int kStaticMaxEntries = 1 << 20;
constexpr int kStaticBlocks = 64;
constexpr int kStaticWarps = kStaticBlocks * (kSchedThreads / 32);
// histogram scan workspace: 64 chunk groups of every key, the key bases, a ticket
constexpr int kStaticScanWords = 64 * kStaticMaxDomains + kStaticMaxDomains + 1;

struct StaticScratch {
  DomainDev domains[kStaticMaxDomains];
  uint32_t list[kStaticMaxRays];
  uint64_t ray_key[kStaticMaxRays];
  uint2 arena[kStaticMaxEntries];
  uint32_t list_off[kStaticMaxRays];
  uint32_t list_cnt[kStaticMaxRays];
  uint32_t hist[kStaticMaxDomains * kStaticWarps];
  long long dstats[kStaticMaxDomains * kMaxList];
  uint32_t scan_tmp[kStaticScanWords];
  unsigned long long arena_top;
  uint32_t count;
  uint32_t num_entries;
  Counters ctr;
};

// The scheduler's scratch, laid out as a StaticScratch: one per device,
// shared by every call.  Host code must not use this name as an address.
static __device__ __align__(256) unsigned char g_sched_scratch[sizeof(StaticScratch)];

// Host copy of the array's device address, per device.
std::mutex g_mutex;
StaticScratch* g_scratch_addr[64] = {nullptr};

__global__ void kStaticPrepare(StaticScratch* s, const float* __restrict__ bounds, int D, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < D) {
    DomainDev d{};
    for (int c = 0; c < 3; ++c) {
      d.bmin[c] = bounds[6 * i + c];
      d.bmax[c] = bounds[6 * i + 3 + c];
    }
    s->domains[i] = d;
  }
  for (int k = i; k < n; k += gridDim.x * blockDim.x) s->list[k] = (uint32_t)k;
  if (i == 0) {
    s->count = (uint32_t)n;
    s->arena_top = 0ull;
    s->num_entries = 0u;
    s->ctr = Counters{};
  }
  for (int k = i; k < D * kMaxList; k += gridDim.x * blockDim.x) s->dstats[k] = 0;
}

}  // namespace
}  // namespace spray

extern "C" int spray_gpu_schedule_static(const float* domain_bounds, int32_t num_domains,
                                         const float* ray_org, const float* ray_dir, int32_t num_rays,
                                         int32_t list_size, uint32_t* entries,
                                         int64_t entry_capacity, uint32_t* domain_start,
                                         int64_t* num_entries, void* stream) {
  using namespace spray;
  try {
  if (!domain_bounds || !ray_org || !ray_dir || !entries || !domain_start || !num_entries)
    return fail(SPRAY_GPU_EINVAL, "null argument");
  if (num_domains <= 0 || num_domains > kStaticMaxDomains)
    return fail(SPRAY_GPU_EINVAL, "num_domains must be in [1, " + std::to_string(kStaticMaxDomains) + "]");
  if (num_rays < 0 || num_rays > kStaticMaxRays)
    return fail(SPRAY_GPU_EINVAL, "num_rays must be in [0, " + std::to_string(kStaticMaxRays) + "]");
  if (list_size <= 0 || list_size > kMaxList) return fail(SPRAY_GPU_EINVAL, "list_size must be in [1, 32]");
  if (entry_capacity < 0) return fail(SPRAY_GPU_EINVAL, "negative entry capacity");
  if ((((uintptr_t)ray_org) | ((uintptr_t)ray_dir) | ((uintptr_t)entries)) & 15u)
    return fail(SPRAY_GPU_EINVAL, "ray and entry arrays must be 16-byte aligned");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(SPRAY_GPU_ECUDA, "device ordinal out of range");
  StaticScratch* s = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_sched_scratch);
      if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = static_cast<StaticScratch*>(p);
    }
    s = g_scratch_addr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int D = num_domains;
  kStaticPrepare<<<(std::max(num_rays, D * kMaxList) + 255) / 256 + 1, 256, 0, st>>>(s, domain_bounds, D,
                                                                                    num_rays);
  SchedArgs a{};
  a.shadow = 0;
  a.count = &s->count;
  a.list = s->list;
  a.rays.org = reinterpret_cast<float4*>(const_cast<float*>(ray_org));
  a.rays.dir = reinterpret_cast<float4*>(const_cast<float*>(ray_dir));
  a.slots = 1;
  a.order_by_depth = 0;
  a.list_size = list_size;
  a.ray_key = s->ray_key;
  a.arena = s->arena;
  a.arena_top = &s->arena_top;
  a.arena_cap = kStaticMaxEntries;
  a.list_off = s->list_off;
  a.list_cnt = s->list_cnt;
  a.hist = s->hist;
  a.nchunks = kStaticWarps;  // one chunk per warp: at most 512 rays, 16-bit counts
  a.pack_depth = 1;  // ray | position << 26 | origin << 31, as the header documents
  a.dstats = s->dstats;
  a.entries = reinterpret_cast<uint2*>(entries);
  a.entry_cap = (unsigned long long)entry_capacity;
  a.key_start = domain_start;
  a.num_entries = &s->num_entries;
  a.ctr = &s->ctr;
  launchSchedule(st, a, s->domains, D, kStaticWarps, kStaticBlocks, s->scan_tmp, kStaticScanWords);
  Counters ctr;
  uint32_t ne = 0;
  e = cudaMemcpyAsync(&ne, &s->num_entries, sizeof(ne), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&ctr, &s->ctr, sizeof(ctr), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(SPRAY_GPU_ECUDA, cudaGetErrorString(e));
  if (ctr.list_overflows) return fail(SPRAY_GPU_EOVERFLOW, "a ray overlapped more than 32 domains");
  if (ctr.arena_overflows) return fail(SPRAY_GPU_EOVERFLOW, "more queue entries than the static scratch holds");
  if (ctr.entry_overflows) return fail(SPRAY_GPU_EOVERFLOW, "entry_capacity too small");
  *num_entries = (int64_t)ne;
  return SPRAY_GPU_OK;
  } catch (const std::exception& ex) {
    // no C++ exception crosses the C boundary (launch configuration errors,
    // allocation failures of the error strings)
    return fail(SPRAY_GPU_ECUDA, ex.what());
  }
}
