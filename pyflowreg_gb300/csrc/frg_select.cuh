// Forgetful selection of the median of two vertically adjacent 5 x 5 windows
// on the float pipe, shared by the float32 median (values) and the float64
// median (float keys of the values).
#pragma once

#include <cuda_runtime.h>

namespace frg {

__device__ __forceinline__ void sel_swap(float& x, float& y)
{
    const float lo = fminf(x, y), hi = fmaxf(x, y);
    x = lo;
    y = hi;
}

// Medians of two 25-element windows that share their first 20 elements
// (vertically adjacent 5 x 5 windows: v[0..19] the four common rows, a[0..4]
// and b[0..4] the rows only one window has).  Forgetful selection: keep 14
// candidates, repeatedly drop the minimum and the maximum and admit the next
// value; the middle of the last three is the 13th smallest.  The rounds that
// only see common elements (the first 14, then v[14..19]) run once for both
// windows; the last four rounds and the final median of three run per window.
// Each result is the median of its window.
__device__ __forceinline__ void median25_pair(const float v[20], const float a[5], const float b[5], float& ma,
                                              float& mb)
{
    float t[14];
#pragma unroll
    for (int i = 0; i < 14; ++i) t[i] = v[i];
#pragma unroll
    for (int round = 0; round < 7; ++round) {
        const int lo = round;
#pragma unroll
        for (int i = lo + 1; i < 14; ++i) sel_swap(t[lo], t[i]);
#pragma unroll
        for (int i = lo + 1; i < 13; ++i) sel_swap(t[i], t[13]);
        t[13] = round < 6 ? v[14 + round] : 0.0f;
    }
    // round 6 dropped t[6] and t[13]; t[7..12] are the shared survivors
    float ta[14], tb[14];
#pragma unroll
    for (int i = 7; i < 13; ++i) ta[i] = tb[i] = t[i];
    ta[13] = a[0];
    tb[13] = b[0];
#pragma unroll
    for (int round = 7; round < 11; ++round) {
        const int lo = round;
#pragma unroll
        for (int i = lo + 1; i < 14; ++i) {
            sel_swap(ta[lo], ta[i]);
            sel_swap(tb[lo], tb[i]);
        }
#pragma unroll
        for (int i = lo + 1; i < 13; ++i) {
            sel_swap(ta[i], ta[13]);
            sel_swap(tb[i], tb[13]);
        }
        ta[13] = a[round - 6];
        tb[13] = b[round - 6];
    }
    sel_swap(ta[11], ta[12]);
    sel_swap(ta[12], ta[13]);
    sel_swap(ta[11], ta[12]);
    sel_swap(tb[11], tb[12]);
    sel_swap(tb[12], tb[13]);
    sel_swap(tb[11], tb[12]);
    ma = ta[12];
    mb = tb[12];
}

}  // namespace frg
