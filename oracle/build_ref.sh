#!/bin/sh
# TEST INFRASTRUCTURE ONLY.  Builds, from the reference's own sources where
# they lie (read-only), the two libraries the oracle is checked against:
#   oracle/_ref/libref_rng.so   deps/embree/random_sampler.h (ref_rng.cpp)
#   oracle/_ref/libref_path.so  render/{sampler,lru_cache,tile,trimesh_buffer}.cc,
#                               ooc/{ooc_domain_stats,ooc_vbuf}.cc,
#                               baseline/baseline_schedulers.cc,
#                               io/{scene_loader,ply_loader}.cc,
#                               deps/pbrt/memory.cpp and the inline code of
#                               render/{aabb,camera,light,reflection}.h,
#                               display/image.h, utils/util.h and render/rays.h
#                               (ref_path.cpp)
# oracle/ref_shim stands in for glm, glog, mpi.h, the CMake-generated config
# header, the MPI profiler header and the Embree 2 declarations, none of which
# exist here.  Nothing of the
# reference is copied.  Exits 0 without building when the reference tree is
# absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${SPRAY_REFERENCE_DIR:-/root/reference}
[ -f "$REF/deps/embree/random_sampler.h" ] || { echo "reference sources absent: oracle/_ref not built"; exit 0; }
mkdir -p "$HERE/_ref"
FLAGS="-O2 -std=c++17 -fPIC -shared -ffp-contract=off -w"
g++ $FLAGS -I "$HERE/ref_shim" -I "$REF/deps/embree" \
    "$HERE/ref_rng.cpp" -o "$HERE/_ref/libref_rng.so"
# the reference's own language level (cmake/pbrt_compile.cmake) and the
# definitions its compiler probes give on Linux/g++ (cmake/pbrt_flags.cmake);
# deps/pbrt's BlockedArray needs -fpermissive with current g++
# (__forceinline: what Embree's platform header defines for random_sampler.h;
# baseline/baseline_ray.h uses INT_MAX without including <climits>)
g++ $FLAGS -std=gnu++11 -fpermissive -include climits -DPBRT_HAVE_CONSTEXPR -DPBRT_CONSTEXPR=constexpr -D__forceinline=inline \
    -DPBRT_HAVE_ALIGNAS -DPBRT_HAVE_ALIGNOF -DPBRT_HAVE_POSIX_MEMALIGN \
    -I "$HERE/ref_shim" -I "$REF/src" -I "$REF/deps" \
    "$HERE/ref_path.cpp" "$REF/src/render/sampler.cc" "$REF/src/render/lru_cache.cc" "$REF/src/render/tile.cc" \
    "$REF/src/render/trimesh_buffer.cc" "$REF/src/baseline/baseline_schedulers.cc" \
    "$REF/src/ooc/ooc_domain_stats.cc" "$REF/src/io/scene_loader.cc" "$REF/src/io/ply_loader.cc" \
    "$REF/src/ooc/ooc_vbuf.cc" "$REF/deps/pbrt/memory.cpp" \
    -o "$HERE/_ref/libref_path.so"
echo "$HERE/_ref/libref_rng.so $HERE/_ref/libref_path.so"
