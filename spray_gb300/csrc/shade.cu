// AO and path-tracing shaders applied to resolved closest hits, and the
// retire step that accumulates unoccluded shadow rays into the image.
//
// The shaders restate ShaderAo::operator() (src/ooc/ooc_shader_ao.h:92-197)
// and ShaderPt::operator() (src/ooc/ooc_shader_pt.h:93-227) for the single
// hit a wavefront keeps per sample: the speculative loop only retires shadow
// rays whose history matches the sample's closest hits
// (src/ooc/ooc_vbuf.cc:41-52, ooc_tcontext.inl:123-135), which are exactly
// the rays spawned here.  Shadow ray `slot` of alive ray a lives at
// a * slots + slot.
#include <algorithm>

#include "kernels.cuh"
#include "shade.cuh"
#include "spray_math.cuh"

namespace spray {

__constant__ float c_unpack[256];  // i * SPRAY_1_OVER_255 rounded to float

namespace {

__device__ __forceinline__ V3 unpackColor(uint32_t c) {
  return v3(c_unpack[(c >> 16) & 0xffu], c_unpack[(c >> 8) & 0xffu], c_unpack[c & 0xffu]);
}

__device__ __forceinline__ void writeShadow(const ShadeArgs& a, uint32_t sid, V3 wi, V3 w, float tmax,
                                            bool valid) {
  if (valid) {
    a.sh.dir[sid] = make_float4(wi.x, wi.y, wi.z, tmax);
    a.sh.wgt[sid] = make_float4(w.x, w.y, w.z, 1.0f);
  }
  a.shadow_flag[sid] = valid ? 1 : 0;
}

__device__ __forceinline__ int domainOfPrim(const DomainDev* doms, int D, uint32_t gprim) {
  int lo = 0, hi = D - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (doms[mid].gprim_base <= gprim) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

}  // namespace

// Domains whose first global face number the shader keeps in shared memory
// for the hit's domain search (more domains search the device table).
constexpr int kShadeSmemDomains = 4096;

// Four resident blocks per SM (64 registers): the shader is latency-bound,
// and occupancy pays more than the few spills (measured against 94 registers).
__global__ void __launch_bounds__(256, 4) kShade(ShadeArgs a) {
  __shared__ uint32_t sprim[kShadeSmemDomains];
  const int D = a.scene.num_domains;
  const bool stab = D <= kShadeSmemDomains;
  if (stab)
    for (int k = threadIdx.x; k < D; k += blockDim.x) sprim[k] = a.scene.domains[k].gprim_base;
  __syncthreads();
  const uint32_t n = *a.count;
  const int S = a.slots;
  const ShadeEnv env{a.lights, a.num_lights, {a.ks[0], a.ks[1], a.ks[2]}, a.shininess, a.ctr};
  unsigned long long nshadow = 0, nbounce = 0;
  // a contiguous range of alive rays per block (the compaction's partition)
  const uint64_t per = ((uint64_t)n + gridDim.x - 1) / gridDim.x;
  const uint64_t i0 = min((uint64_t)n, per * blockIdx.x), i1 = min((uint64_t)n, i0 + per);
  for (uint64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const uint32_t sample = a.list[i];
    const uint64_t key = a.ray_key[sample];
    a.next_flag[sample] = 0;  // set below when a bounce ray is emitted
    const uint32_t sbase = (uint32_t)i * S;
    if (key == kNoHit) {
      for (int s = 0; s < S; ++s) a.shadow_flag[sbase + s] = 0;
      continue;
    }
    const float t = hitKeyT(key);
    // the sample's loads first: they do not depend on the domain search
    // primary rays (depth 0) carry weight 1, which kGenPrimary does not store
    const float4 o4 = a.rays.org[sample], d4 = a.rays.dir[sample];
    const float4 w4 = a.depth == 0 ? make_float4(1.f, 1.f, 1.f, 0.f) : a.rays.wgt[sample];
    const float4 hn = a.hit_ns[sample];
    int d;
    if (stab) {
      // last domain whose first global face is <= the hit's
      const uint32_t gprim = (uint32_t)key;
      int lo = 0, hi = D - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sprim[mid] <= gprim) lo = mid;
        else hi = mid - 1;
      }
      d = lo;
    } else {
      d = domainOfPrim(a.scene.domains, D, (uint32_t)key);
    }
    const DomainDev dom = a.scene.domains[d];
    const V3 org = v3(o4.x, o4.y, o4.z), dir = v3(d4.x, d4.y, d4.z);
    const V3 Lin = v3(w4.x, w4.y, w4.z);
    const V3 pos = v3(dir.x * t + org.x, dir.y * t + org.y, dir.z * t + org.z);
    const V3 normal = v3(hn.x, hn.y, hn.z);
    const V3 surf = unpackColor(__float_as_uint(hn.w));
    const int pixid = a.rays.pixid[sample];
    const int samid = a.rays.samid[sample];
    const ViewDev& vw = a.views[a.rays.view[sample]];
    a.sh.hitpos[i] = make_float4(pos.x, pos.y, pos.z, __int_as_float(d));
    const int used = shadeHit(
        env, vw, dir, Lin, pos, normal, surf, dom.bsdf, dom.bsdf_p, pixid, samid, a.depth + 1,
        [&](int slot, V3 wi, V3 w, float tmax, bool valid) {
          writeShadow(a, sbase + slot, wi, w, tmax, valid);
          nshadow += valid;
        },
        [&](V3 wi, V3 w) {
          // bounce ray (genR2); the speculation-history wrap of the reference
          // (pending queue at SPRAY_HISTORY_SIZE) does not change the depth count
          a.next.org[sample] = make_float4(pos.x, pos.y, pos.z, 0.f);
          a.next.dir[sample] = make_float4(wi.x, wi.y, wi.z, 0.f);
          a.next.wgt[sample] = make_float4(w.x, w.y, w.z, 0.f);
          a.next_flag[sample] = 1;
          ++nbounce;
        });
    for (int slot = used; slot < S; ++slot) a.shadow_flag[sbase + slot] = 0;
  }
  for (int o = 16; o; o >>= 1) {
    nshadow += __shfl_down_sync(0xffffffffu, nshadow, o);
    nbounce += __shfl_down_sync(0xffffffffu, nbounce, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (nshadow) atomicAdd(&a.ctr->rays_shadow, nshadow);
    if (nbounce) atomicAdd(&a.ctr->rays_bounce, nbounce);
  }
  if (a.blk_shadow) {
    // this block's kept counts for the two compactions that follow
    __shared__ unsigned int bsum[2];
    if (threadIdx.x == 0) bsum[0] = bsum[1] = 0u;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&bsum[0], (unsigned int)nshadow);
      atomicAdd(&bsum[1], (unsigned int)nbounce);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      a.blk_shadow[blockIdx.x] = bsum[0];
      a.blk_next[blockIdx.x] = bsum[1];
    }
  }
}

void initShadeTables() {
  float lut[256];
  for (int i = 0; i < 256; ++i) lut[i] = (float)(i * kOneOver255);
  cudaMemcpyToSymbol(c_unpack, lut, sizeof(lut));
}

void launchShade(cudaStream_t s, const ShadeArgs& a, int nblocks) {
  kShade<<<nblocks, 256, 0, s>>>(a);
}

// Retire (CommitBuffer::retire, src/ooc/ooc_tcontext.inl:123-135, with
// HdrImage::add, src/display/image.h:99-109): per pixel, its samples in order,
// each sample's slots in order, every unoccluded shadow ray adds w * (1 / spp)
// in double precision.
//
// Only the pixels with a sample alive at this depth can receive anything, so
// the kernel walks the depth's alive list (samples in order; a pixel's samples
// are consecutive sample ids s0 .. s0 + spp - 1, s0 = s - samid % spp).  A warp
// takes the list 32 entries at a time and queues the entries that start a
// pixel (the previous entry lies before s0) in a per-warp FIFO; once 32 wait
// (or the list ends) every lane adds one pixel's contributions.  The alive
// index of an entry is its position in the list, so shadow slot k of entry j
// is j * S + k.
__device__ __forceinline__ void retirePixel(float4* image, const ViewDev* __restrict__ views,
                                            const uint32_t* __restrict__ list, uint32_t n, uint32_t j,
                                            const RayBuf& rays, const ShadowBuf& sh,
                                            const uint8_t* __restrict__ flag, int S) {
  const uint32_t s = list[j];
  const ViewDev& vw = views[rays.view[s]];
  const uint32_t send = s - (uint32_t)(rays.samid[s] % vw.spp) + (uint32_t)vw.spp;
  float4* px = image + vw.pixel_base + rays.pixid[s];
  const double scale = vw.scale;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  bool touched = false;
  for (uint32_t q = j; q < n; ++q) {
    if (q > j && list[q] >= send) break;
    for (int k = 0; k < S; ++k) {
      const uint32_t sid = q * (uint32_t)S + (uint32_t)k;
      if (!flag[sid] || sh.occluded[sid]) continue;
      const float4 w = sh.wgt[sid];
      if (!touched) acc = *px;
      acc.x = (float)((double)acc.x + scale * (double)w.x);
      acc.y = (float)((double)acc.y + scale * (double)w.y);
      acc.z = (float)((double)acc.z + scale * (double)w.z);
      touched = true;
    }
  }
  if (touched) *px = acc;
}

__global__ void __launch_bounds__(256) kRetire(float4* image, const ViewDev* __restrict__ views,
                                               const uint32_t* __restrict__ list,
                                               const uint32_t* __restrict__ count, RayBuf rays, ShadowBuf sh,
                                               const uint8_t* __restrict__ flag, int S) {
  __shared__ uint32_t fifo[8][64];
  uint32_t* q = fifo[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  uint32_t below;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(below));
  const uint32_t n = *count;
  const uint32_t nchunks = (n + 31u) >> 5;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  int nq = 0;
  for (uint32_t c = warp;; c += nwarps) {
    const bool more = c < nchunks;
    if (more) {
      const uint32_t j = (c << 5) + lane;
      bool head = false;
      if (j < n) {
        const uint32_t s = list[j];
        const uint32_t s0 = s - (uint32_t)(rays.samid[s] % views[rays.view[s]].spp);
        head = j == 0 || list[j - 1] < s0;
      }
      const uint32_t hm = __ballot_sync(0xffffffffu, head);
      if (head) q[nq + __popc(hm & below)] = j;  // nq < 32 here, so at most 63 queued
      nq += __popc(hm);
      __syncwarp();
    }
    while (nq >= 32 || (!more && nq > 0)) {
      const int take = min(nq, 32), rest = nq - take;
      if (lane < take) retirePixel(image, views, list, n, q[lane], rays, sh, flag, S);
      const uint32_t moved = lane < rest ? q[take + lane] : 0u;
      __syncwarp();
      if (lane < rest) q[lane] = moved;
      __syncwarp();
      nq = rest;
    }
    if (!more) break;
  }
}

void launchRetire(cudaStream_t s, float4* image, const ViewDev* views, const uint32_t* list, const uint32_t* count,
                  const RayBuf& rays, const ShadowBuf& sh, const uint8_t* flag, int slots, int nblocks) {
  kRetire<<<nblocks, 256, 0, s>>>(image, views, list, count, rays, sh, flag, slots);
}

}  // namespace spray
