// Device helpers shared by the query kernels (hc_query.cu) and the learned
// e-value tail (hc_mlp.cu). Not installed; not part of the C ABI.
#pragma once

#include <cstdint>

namespace hc {

// histogram bin of a hyperscore, (int)(h * 10 + 0.5) as the reference writes
// it (dslim_query.cpp:712, 778): a float product, then a double sum
__device__ __forceinline__ int hist_bin(float hf)
{
    const float t = __fmul_rn(hf, 10.0f);
    return (int)__dadd_rn((double)t, 0.5);
}

// cvttsd2si semantics of the reference's double -> int conversions
// (expeRT.cpp:703-704): out-of-range and NaN give INT_MIN
__device__ __forceinline__ int32_t x86_d2i(double v)
{
    if (!(v > -2147483649.0 && v < 2147483648.0)) return (int32_t)0x80000000u;
    return (int32_t)v;
}

// The tail-fit bins of a spectrum (expeRT.cpp:590-601), by one warp:
// end1 = last bin below the top hit's bin `hyp` holding a candidate, stt1 =
// the first such bin, end1 moved one up when they coincide. Bins past the
// histogram (the reference writes there only out of bounds) read as empty.
// Returns the number of points, end1 - stt1 + 1 (clamped to the histogram).
__device__ __forceinline__ int tail_bins(const uint32_t *__restrict__ yy, int hyp, int nbins, int lane, int &stt1,
                                         int &end1)
{
    end1 = hyp - 1;
    for (int q0 = min(hyp - 1, nbins - 1); q0 >= 0; q0 -= 32)
    {
        const int q = q0 - lane;
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, q >= 0 && yy[q] >= 1u);
        if (b)
        {
            end1 = q0 - (__ffs(b) - 1);
            break;
        }
    }
    stt1 = 0;
    for (int q0 = 0; q0 <= end1 && q0 < nbins; q0 += 32)
    {
        const int q = q0 + lane;
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, q <= end1 && q < nbins && yy[q] >= 1u);
        if (b)
        {
            stt1 = q0 + __ffs(b) - 1;
            break;
        }
    }
    if (stt1 == end1) end1 += 1;
    int n = end1 - stt1 + 1;
    if (n < 0) n = 0;
    if (stt1 + n > nbins) n = nbins - stt1;
    return n;
}

}  // namespace hc
