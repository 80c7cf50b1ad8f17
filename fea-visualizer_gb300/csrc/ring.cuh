// ring.cuh -- pieces shared by the CG iteration kernels that stream the
// operator through a ring of shared-memory stages (single-mesh variants 14
// and 15, the batched variant 14) and load the row vectors directly: cache-
// hinted global loads, the halo slot of a thread, and the stage layout.
#pragma once

#include <stdint.h>
#include <string.h>

#include "cg_device.cuh"

namespace fea {
namespace {

// Loads of data read once per iteration (the operator entries and columns):
// no L1 allocation, first out of the L2 (policy from l2_evict_first_policy).
template <typename T>
__device__ __forceinline__ T ld_once(const T* p, uint64_t pol) {
    T o;
    if constexpr (sizeof(T) == 4) {
        uint32_t x;
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(x) : "l"(p), "l"(pol));
        memcpy(&o, &x, 4);
    } else if constexpr (sizeof(T) == 8) {
        uint2 x;
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.b32 {%0, %1}, [%2], %3;"
            : "=r"(x.x), "=r"(x.y)
            : "l"(p), "l"(pol));
        memcpy(&o, &x, 8);
    } else {
        static_assert(sizeof(T) == 16, "4, 8 or 16 bytes");
        uint4 x;
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.b32 {%0, %1, %2, %3}, [%4], %5;"
            : "=r"(x.x), "=r"(x.y), "=r"(x.z), "=r"(x.w)
            : "l"(p), "l"(pol));
        memcpy(&o, &x, 16);
    }
    return o;
}
__device__ __forceinline__ uint32_t ld_once_u16(const uint16_t* p, uint64_t pol) {
    unsigned short x;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(x) : "l"(p), "l"(pol));
    return x;
}
// Loads of the iteration's vectors, which the next iteration reads again:
// kept in the L2 ahead of the operator (l2_evict_last_policy).
template <typename T>
__device__ __forceinline__ T ld_keep(const T* p, uint64_t pol) {
    T o;
    if constexpr (sizeof(T) == 4) {
        uint32_t x;
        asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(x) : "l"(p), "l"(pol));
        memcpy(&o, &x, 4);
    } else if constexpr (sizeof(T) == 8) {
        uint2 x;
        asm volatile("ld.global.nc.L2::cache_hint.v2.b32 {%0, %1}, [%2], %3;"
                     : "=r"(x.x), "=r"(x.y)
                     : "l"(p), "l"(pol));
        memcpy(&o, &x, 8);
    } else {
        static_assert(sizeof(T) == 16, "4, 8 or 16 bytes");
        uint4 x;
        asm volatile("ld.global.nc.L2::cache_hint.v4.b32 {%0, %1, %2, %3}, [%4], %5;"
                     : "=r"(x.x), "=r"(x.y), "=r"(x.z), "=r"(x.w)
                     : "l"(p), "l"(pol));
        memcpy(&o, &x, 16);
    }
    return o;
}

// Thread t's halo slot: slots are dealt round-robin over the warps, so every
// warp stages about the same share of a tile's halo.
__device__ __forceinline__ int halo_slot(int t) { return (t & 7) * 32 + (t >> 3); }

// One stage of the ring: a tile's operator entries, then (mv > 0) its mass
// entries of mv bytes each, then its local columns.
struct RingStage {
    size_t A, M, L, bytes;
    __host__ __device__ RingStage(int emax, size_t fv, size_t mv = 0) {
        auto al = [](size_t x) { return (x + 127) & ~(size_t)127; };
        A = 0;
        M = al(fv * (size_t)emax);
        L = al(M + mv * (size_t)emax);
        bytes = al(L + 2 * (size_t)emax);
    }
};

// Dynamic shared memory of the single-mesh ring kernels: the ring (which the
// end-of-launch reduction reuses once every copy has landed); the two u'
// buffers follow it.  mv: bytes of a mass entry in the stages (0: none).
template <typename R, int NF>
__host__ __device__ size_t ring_bytes(int emax, int stages, size_t mv = 0) {
    const size_t ring = (size_t)stages * RingStage(emax, sizeof(FV<R, NF>), mv).bytes;
    const size_t red = (size_t)3 * NF * kBlock * sizeof(typename Acc<R>::Packed);
    return (ring > red ? ring : red + 127) & ~(size_t)127;
}

}  // namespace
}  // namespace fea
