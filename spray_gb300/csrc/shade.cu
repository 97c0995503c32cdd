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

// Per pixel of the wave: samples in order, slots in order, each unoccluded
// shadow ray adds w * (1 / spp) with the double-precision scale of
// HdrImage::add (src/display/image.h:99-109).
// Per pixel of the wave: its tile (binary search on pix_base), its samples
// (tile-local pixel lp holds samples lp * spp .. lp * spp + spp - 1), its view's
// image slot and scale; samples and slots in order, the sum in double.
//
// A block takes 256 consecutive pixels, whose samples are one contiguous
// range: their alive indices are staged in shared memory with coalesced loads
// (one pad word per 32, so that each thread's run of spp indices is read
// without bank conflicts) when the range fits kRetireStage, else read directly.
constexpr int kRetireStage = 4096;

__global__ void __launch_bounds__(256) kRetire(float4* image, const TileDev* __restrict__ tiles, int ntiles,
                                               int64_t npix, const ViewDev* __restrict__ views,
                                               const int32_t* __restrict__ alive_idx, ShadowBuf sh,
                                               const uint8_t* __restrict__ flag, int S) {
  __shared__ int32_t sidx[kRetireStage + kRetireStage / 32];
  __shared__ int64_t range[2];
  for (int64_t p0 = (int64_t)blockIdx.x * blockDim.x; p0 < npix; p0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = p0 + threadIdx.x;
    const bool valid = p < npix;
    int lo = 0;
    if (valid) {
      int hi = ntiles - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tiles[mid].pix_base <= p) lo = mid;
        else hi = mid - 1;
      }
    }
    const TileDev tl = tiles[lo];
    const int spp = tl.spp;
    const int64_t lp = p - tl.pix_base;
    const int64_t s0 = tl.sample_base + lp * spp;
    if (threadIdx.x == 0) range[0] = s0;
    if (p == min(npix, p0 + (int64_t)blockDim.x) - 1) range[1] = s0 + spp;
    __syncthreads();
    const int64_t sbeg = range[0], nstage = range[1] - range[0];
    const bool staged = nstage <= kRetireStage;
    if (staged) {
      // 8 loads in flight per thread before their shared-memory stores
      for (int j0 = threadIdx.x; j0 < (int)nstage; j0 += 8 * blockDim.x) {
        int32_t v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int j = j0 + u * (int)blockDim.x;
          v[u] = j < (int)nstage ? alive_idx[sbeg + j] : 0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int j = j0 + u * (int)blockDim.x;
          if (j < (int)nstage) sidx[j + (j >> 5)] = v[u];
        }
      }
    }
    __syncthreads();
    if (valid) {
      const ViewDev& vw = views[tl.view];
      const double scale = vw.scale;
      const int lpi = (int)lp;  // tile-local pixel (32-bit division)
      const int x = tl.x + lpi % tl.w, y = tl.y + lpi / tl.w;
      float4* px = image + vw.pixel_base + (int64_t)y * vw.image_w + x;
      float4 acc = *px;
      bool touched = false;
      const int f0 = (int)(s0 - sbeg);
      for (int s = 0; s < spp; ++s) {
        const int f = f0 + s;
        const int32_t ai = staged ? sidx[f + (f >> 5)] : alive_idx[s0 + s];
        if (ai < 0) continue;
        for (int k = 0; k < S; ++k) {
          uint32_t sid = (uint32_t)ai * S + k;
          if (!flag[sid] || sh.occluded[sid]) continue;
          float4 w = sh.wgt[sid];
          acc.x = (float)((double)acc.x + scale * (double)w.x);
          acc.y = (float)((double)acc.y + scale * (double)w.y);
          acc.z = (float)((double)acc.z + scale * (double)w.z);
          touched = true;
        }
      }
      if (touched) *px = acc;
    }
    __syncthreads();  // the next group restages sidx and range
  }
}

void launchRetireImpl(cudaStream_t s, float4* image, const TileDev* tiles, int ntiles, int64_t npix,
                      const ViewDev* views, const int32_t* alive_idx, const ShadowBuf sh,
                      const uint8_t* flag, int slots, int nblocks) {
  // one 256-pixel group per block where the grid allows (the staged loads of
  // many blocks overlap), at least nblocks
  const int64_t groups = (npix + 255) / 256;
  const int64_t blocks = std::max<int64_t>(nblocks, std::min<int64_t>(groups, 1 << 24));
  kRetire<<<(unsigned)blocks, 256, 0, s>>>(image, tiles, ntiles, npix, views, alive_idx, sh, flag, slots);
}

}  // namespace spray
