// lss_select.cuh -- the per-sample median across channels (the common-average reference).
//
// A warp holds one sample's C channel values, NJ per lane, as order-preserving unsigned keys
// (float_key: negative values bit-inverted, non-negative ones with the sign bit set, so unsigned
// order is float order).  warp_kth_smallest finds the k-th smallest key (0-based) by a binary
// search on the key value, most significant bit first: each pass counts the keys below
// prefix + 2^bit (one compare and one add per key, one warp reduction) and keeps the half that
// holds rank k.  It stops as soon as a single key lies in the remaining interval -- about
// log2(C) + a few passes for distinct values instead of 32 -- and runs to bit 0 on ties, where
// the interval's lower end is the answer.  Padding keys are 0xffffffff (never counted below any
// threshold), so k < the number of real keys is required.
#pragma once

#include <cstdint>

namespace lss {

__device__ __forceinline__ uint32_t float_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

template <int NJ>
__device__ __forceinline__ uint32_t warp_kth_smallest(const uint32_t (&key)[NJ], int k) {
    uint32_t lo = 0;           // the answer lies in [lo, lo + 2^(bit+1))
    int below = 0;             // keys < lo
    int alive = 32 * NJ;       // keys in [lo, lo + 2^(bit+1))
    for (int bit = 31; bit >= 0; --bit) {
        const uint32_t mid = lo + (1u << bit);   // lo has zeros at bit and below: no overflow
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < NJ; ++j) cnt += key[j] < mid;
        cnt = __reduce_add_sync(0xffffffffu, cnt);   // keys < mid
        if (k < cnt) {
            alive = cnt - below;
        } else {
            alive -= cnt - below;
            below = cnt;
            lo = mid;
        }
        if (alive == 1) {
            // the one key in [lo, lo + 2^bit)
            uint32_t got = 0;
#pragma unroll
            for (int j = 0; j < NJ; ++j)
                if (key[j] - lo < (1u << bit)) got = key[j];
            return __reduce_or_sync(0xffffffffu, got);
        }
    }
    return lo;
}

}  // namespace lss
