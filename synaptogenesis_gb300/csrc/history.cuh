// Output history shifts shared by the neural models (state/attributes.h:
// 316-333): BIT layers keep 32 steps per word, newest in bit 31, and carry
// the oldest bit of each word into the next; FLOAT layers keep one step per
// word.
#pragma once
#include <cstdint>

namespace sg {

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t shift_bits(uint32_t* out, int size, int history, int nid,
                                               uint32_t new_bit) {
    uint32_t curr = out[(size_t)size * (history - 1) + nid];
    for (int idx = history - 1; idx > 0; --idx) {
        uint32_t prev = out[(size_t)size * (idx - 1) + nid];
        out[(size_t)size * idx + nid] = (curr >> 1) | (prev << 31);
        curr = prev;
    }
    out[nid] = (curr >> 1) | (new_bit << 31);
    return curr >> 31;
}

__device__ __forceinline__ void shift_floats(float* out, int size, int history, int nid, float v) {
    for (int idx = history - 1; idx > 0; --idx)
        out[(size_t)size * idx + nid] = out[(size_t)size * (idx - 1) + nid];
    out[nid] = v;
}
#endif

}  // namespace sg
