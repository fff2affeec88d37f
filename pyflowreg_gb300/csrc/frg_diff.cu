// Differentiable mode: forward kernels and their hand-written adjoints.
//
// The differentiable mode is pyflowreg's flow path with the reference torch
// backend's red-black level solver (torch/core/level_solver.py:11-199) and a
// continuous warp (the reference's cv2.remap rounds map coordinates to 1/32 px,
// core/warping.py:160-234, which has a zero derivative).  Every kernel is
// templated on the arithmetic type T (float or double) and works on planar
// row-major arrays: images (F, K, h, w), flows and solver states (F, 2, h, w)
// with plane 0 = u / du and plane 1 = v / dv.  The solver keeps only the
// interior of the reference's padded arrays; its border copies
// (set_boundary_2d) become clamped neighbour indices.
//
// Adjoints are exact for the unrolled computation: each red-black half-sweep
// is reversed by a gather over the same stencil with the same coefficients,
// each psi tick by the derivative of psi = a (E + eps)^(a - 1), the motion
// tensor by its local derivative followed by the transposed difference
// stencils, the warp by an atomic scatter of the cubic weights plus the
// derivative of the interpolant, the resizes by their transposed tap tables.
#include <cuda_runtime.h>

#include <cstdint>

#include "frg_internal.h"

namespace frg {
namespace diff {

namespace {

__device__ __forceinline__ int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }

template <typename T>
__device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }

// Keys cubic convolution (R. Keys, 1981), A = -0.75: weights of the taps at
// offsets -1, 0, 1, 2 for a fraction t in [0, 1), in the Horner form the
// oracle uses, and their derivatives in t.
template <typename T>
__device__ __forceinline__ void keys4(T t, T w[4])
{
    const T a = (T)-0.75;
    const T s = t + (T)1;
    w[0] = ((a * s - (T)5 * a) * s + (T)8 * a) * s - (T)4 * a;
    w[1] = ((a + (T)2) * t - (a + (T)3)) * t * t + (T)1;
    const T r = (T)1 - t;
    w[2] = ((a + (T)2) * r - (a + (T)3)) * r * r + (T)1;
    const T q = (T)2 - t;
    w[3] = ((a * q - (T)5 * a) * q + (T)8 * a) * q - (T)4 * a;
}

template <typename T>
__device__ __forceinline__ void dkeys4(T t, T d[4])
{
    const T a = (T)-0.75;
    const T s = t + (T)1;
    d[0] = (T)3 * a * s * s - (T)10 * a * s + (T)8 * a;
    d[1] = (T)3 * (a + (T)2) * t * t - (T)2 * (a + (T)3) * t;
    const T r = (T)1 - t;
    d[2] = -((T)3 * (a + (T)2) * r * r - (T)2 * (a + (T)3) * r);
    const T q = (T)2 - t;
    d[3] = -((T)3 * a * q * q - (T)10 * a * q + (T)8 * a);
}

template <typename T>
__device__ __forceinline__ T tfloor(T x);
template <>
__device__ __forceinline__ float tfloor<float>(float x) { return floorf(x); }
template <>
__device__ __forceinline__ double tfloor<double>(double x) { return floor(x); }

template <typename T>
__device__ __forceinline__ T tpow(T x, T y);
template <>
__device__ __forceinline__ float tpow<float>(float x, float y) { return powf(x, y); }
template <>
__device__ __forceinline__ double tpow<double>(double x, double y) { return pow(x, y); }

template <typename T>
__device__ __forceinline__ void atomic_add(T* p, T v) { atomicAdd(p, v); }

// ------------------------------------------------------------------ resize
// Horizontal pass of the separable resample (util/resize_util.py:116-141):
// dst(p, y, x) = sum_t wx[x, t] * src(p, y, ix[x, t]).
template <typename T>
__global__ void kd_resize_h(const T* __restrict__ src, int ih, int iw, int ow, const int32_t* __restrict__ ix,
                            const float* __restrict__ wx, int P, T* __restrict__ dst)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= ow) return;
    const long long row = (long long)blockIdx.z * ih + blockIdx.y;
    const T* s = src + row * iw;
    T acc = 0;
    for (int t = 0; t < P; ++t) acc += (T)wx[x * P + t] * s[ix[x * P + t]];
    dst[row * ow + x] = acc;
}

// Vertical pass: dst(p, y, x) = sum_t wy[y, t] * src(p, iy[y, t], x).
template <typename T>
__global__ void kd_resize_v(const T* __restrict__ src, int ih, int ow, int oh, const int32_t* __restrict__ iy,
                            const float* __restrict__ wy, int P, T* __restrict__ dst)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= ow) return;
    const int y = blockIdx.y;
    const long long p = blockIdx.z;
    const T* s = src + p * ih * (long long)ow;
    T acc = 0;
    for (int t = 0; t < P; ++t) acc += (T)wy[y * P + t] * s[(long long)iy[y * P + t] * ow + x];
    dst[(p * oh + y) * (long long)ow + x] = acc;
}

// Transposed horizontal pass through the inverse (CSR) table of the forward
// taps: g_src(p, y, a) (+)= sum_{e in row a} w[e] * g_dst(p, y, idx[e]).
template <typename T>
__global__ void kd_resize_ht(const T* __restrict__ gdst, int ih, int ow, int iw, const int32_t* __restrict__ ptr,
                             const int32_t* __restrict__ idx, const float* __restrict__ w, T* __restrict__ gsrc,
                             int accumulate)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= iw) return;
    const long long row = (long long)blockIdx.z * ih + blockIdx.y;
    const T* g = gdst + row * ow;
    T acc = 0;
    for (int e = ptr[a]; e < ptr[a + 1]; ++e) acc += (T)w[e] * g[idx[e]];
    T* o = gsrc + row * iw + a;
    *o = accumulate ? *o + acc : acc;
}

// Transposed vertical pass: g_src(p, b, x) = sum_{e in row b} w[e] * g_dst(p, idx[e], x).
template <typename T>
__global__ void kd_resize_vt(const T* __restrict__ gdst, int oh, int ow, int ih, const int32_t* __restrict__ ptr,
                             const int32_t* __restrict__ idx, const float* __restrict__ w, T* __restrict__ gsrc)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= ow) return;
    const int b = blockIdx.y;
    const long long p = blockIdx.z;
    const T* g = gdst + p * oh * (long long)ow;
    T acc = 0;
    for (int e = ptr[b]; e < ptr[b + 1]; ++e) acc += (T)w[e] * g[(long long)idx[e] * ow + x];
    gsrc[(p * ih + b) * (long long)ow + x] = acc;
}

// ------------------------------------------------------------------ warp
// Continuous backward warp (core/warping.py:160-234 without the 1/32 px
// rounding): out(y, x) = f2(y + v / h_row, x + u / h_col) by the Keys cubic
// with replicated borders; pixels whose map leaves [0, w) x [0, h) take f1.
template <typename T>
__global__ void kd_warp(const T* __restrict__ f2, const T* __restrict__ f1, const T* __restrict__ uv, int K, int h,
                        int w, T hcol, T hrow, T* __restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long f = blockIdx.z, hw = (long long)h * w, pix = (long long)y * w + x;
    const T* up = uv + f * 2 * hw;
    const T mx = (T)x + up[pix] / hcol;
    const T my = (T)y + up[hw + pix] / hrow;
    const bool oob = mx < (T)0 || mx >= (T)w || my < (T)0 || my >= (T)h;
    const T mxc = mx < (T)0 ? (T)0 : (mx > (T)(w - 1) ? (T)(w - 1) : mx);
    const T myc = my < (T)0 ? (T)0 : (my > (T)(h - 1) ? (T)(h - 1) : my);
    const T x0 = tfloor(mxc), y0 = tfloor(myc);
    T wx[4], wy[4];
    keys4(mxc - x0, wx);
    keys4(myc - y0, wy);
    int xs[4], ys[4];
    for (int j = 0; j < 4; ++j) xs[j] = clampi((int)x0 + j - 1, 0, w - 1);
    for (int i = 0; i < 4; ++i) ys[i] = clampi((int)y0 + i - 1, 0, h - 1);
    for (int k = 0; k < K; ++k) {
        const long long pl = (f * K + k) * hw;
        if (oob) {
            out[pl + pix] = f1[pl + pix];
            continue;
        }
        T acc = 0;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) acc = acc + (wy[i] * wx[j]) * f2[pl + (long long)ys[i] * w + xs[j]];
        out[pl + pix] = acc;
    }
}

// Adjoint of kd_warp: g_f2 receives the cubic weights by atomic scatter,
// g_f1 the out-of-bounds pixels, g_uv the derivative of the interpolant in
// the map coordinate (zero where the map was clamped to w-1 / h-1).
template <typename T>
__global__ void kd_warp_adj(const T* __restrict__ f2, const T* __restrict__ uv, const T* __restrict__ gout, int K,
                            int h, int w, T hcol, T hrow, T* __restrict__ gf2, T* __restrict__ gf1,
                            T* __restrict__ guv)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long f = blockIdx.z, hw = (long long)h * w, pix = (long long)y * w + x;
    const T* up = uv + f * 2 * hw;
    const T mx = (T)x + up[pix] / hcol;
    const T my = (T)y + up[hw + pix] / hrow;
    const bool oob = mx < (T)0 || mx >= (T)w || my < (T)0 || my >= (T)h;
    if (oob) {
        if (gf1)
            for (int k = 0; k < K; ++k) {
                const long long pl = (f * K + k) * hw;
                gf1[pl + pix] += gout[pl + pix];
            }
        return;
    }
    const bool x_in = mx <= (T)(w - 1), y_in = my <= (T)(h - 1);
    const T mxc = x_in ? mx : (T)(w - 1);
    const T myc = y_in ? my : (T)(h - 1);
    const T x0 = tfloor(mxc), y0 = tfloor(myc);
    T wx[4], wy[4], dx[4], dy[4];
    keys4(mxc - x0, wx);
    keys4(myc - y0, wy);
    dkeys4(mxc - x0, dx);
    dkeys4(myc - y0, dy);
    int xs[4], ys[4];
    for (int j = 0; j < 4; ++j) xs[j] = clampi((int)x0 + j - 1, 0, w - 1);
    for (int i = 0; i < 4; ++i) ys[i] = clampi((int)y0 + i - 1, 0, h - 1);
    T gu = 0, gv = 0;
    for (int k = 0; k < K; ++k) {
        const long long pl = (f * K + k) * hw;
        const T g = gout[pl + pix];
        if (g == (T)0) continue;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                const long long o = pl + (long long)ys[i] * w + xs[j];
                const T s = f2[o];
                atomic_add(gf2 + o, (wy[i] * wx[j]) * g);
                gu += (wy[i] * dx[j]) * s * g;
                gv += (dy[i] * wx[j]) * s * g;
            }
    }
    if (!guv) return;
    T* gp = guv + f * 2 * hw;
    if (x_in) gp[pix] += gu / hcol;
    if (y_in) gp[hw + pix] += gv / hrow;
}

// ------------------------------------------------------------------ motion tensor
// Gradient-constancy terms (core/optical_flow.py:73-160) at pixel (y, x) of
// one channel, through S = (f1 + f2) / 2 and D = f2 - f1 with clamped
// neighbours (the reference's symmetric pads).
template <typename T>
struct GcTerms {
    T a, b, c, p, q;  // fxx, fxy, fyy, fxt, fyt
};

template <typename T>
__device__ __forceinline__ GcTerms<T> gc_terms(const T* __restrict__ f1, const T* __restrict__ f2, int h, int w,
                                               int y, int x, T hy, T hx)
{
    const int xm = x > 0 ? x - 1 : 0, xp = x < w - 1 ? x + 1 : w - 1;
    const int ym = y > 0 ? y - 1 : 0, yp = y < h - 1 ? y + 1 : h - 1;
    auto S = [&](int yy, int xx) {
        const long long o = (long long)yy * w + xx;
        return (T)0.5 * (f1[o] + f2[o]);
    };
    auto Dd = [&](int yy, int xx) {
        const long long o = (long long)yy * w + xx;
        return f2[o] - f1[o];
    };
    const T sc = S(y, x);
    GcTerms<T> r;
    r.a = (S(y, xm) - (T)2 * sc + S(y, xp)) / (hx * hx);
    r.c = (S(ym, x) - (T)2 * sc + S(yp, x)) / (hy * hy);
    const T fxp = (S(yp, xp) - S(yp, xm)) / ((T)2 * hx);
    const T fxm = (S(ym, xp) - S(ym, xm)) / ((T)2 * hx);
    r.b = (fxp - fxm) / ((T)2 * hy);
    r.p = (Dd(y, xp) - Dd(y, xm)) / ((T)2 * hx);
    r.q = (Dd(yp, x) - Dd(ym, x)) / ((T)2 * hy);
    return r;
}

// J (F, 6, K, h, w): J11, J22, J33, J12, J13, J23 of each channel.
template <typename T>
__global__ void kd_tensor(const T* __restrict__ f1, const T* __restrict__ f2, int K, int h, int w, T hy, T hx,
                          T* __restrict__ J)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long fk = blockIdx.z, hw = (long long)h * w, pix = (long long)y * w + x;
    const long long f = fk / K, k = fk % K;
    const GcTerms<T> t = gc_terms(f1 + fk * hw, f2 + fk * hw, h, w, y, x, hy, hx);
    const T rx = (T)1 / (t.a * t.a + t.b * t.b + (T)1e-6);
    const T ry = (T)1 / (t.b * t.b + t.c * t.c + (T)1e-6);
    T* o = J + (f * 6 * K + k) * hw + pix;
    const long long qs = (long long)K * hw;
    o[0 * qs] = rx * t.a * t.a + ry * t.b * t.b;
    o[1 * qs] = rx * t.b * t.b + ry * t.c * t.c;
    o[2 * qs] = rx * t.p * t.p + ry * t.q * t.q;
    o[3 * qs] = rx * t.a * t.b + ry * t.b * t.c;
    o[4 * qs] = rx * t.a * t.p + ry * t.b * t.q;
    o[5 * qs] = rx * t.b * t.p + ry * t.c * t.q;
}

// Local part of the tensor adjoint: from g_J to the gradients of
// (fxx, fxy, fyy, fxt, fyt), stored as G (F, K, 5, h, w).
template <typename T>
__global__ void kd_tensor_adj_local(const T* __restrict__ f1, const T* __restrict__ f2, const T* __restrict__ gJ,
                                    int K, int h, int w, T hy, T hx, T* __restrict__ G)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long fk = blockIdx.z, hw = (long long)h * w, pix = (long long)y * w + x;
    const long long f = fk / K, k = fk % K;
    const GcTerms<T> t = gc_terms(f1 + fk * hw, f2 + fk * hw, h, w, y, x, hy, hx);
    const T rx = (T)1 / (t.a * t.a + t.b * t.b + (T)1e-6);
    const T ry = (T)1 / (t.b * t.b + t.c * t.c + (T)1e-6);
    const T* g = gJ + (f * 6 * K + k) * hw + pix;
    const long long qs = (long long)K * hw;
    const T g11 = g[0], g22 = g[qs], g33 = g[2 * qs], g12 = g[3 * qs], g13 = g[4 * qs], g23 = g[5 * qs];
    const T a = t.a, b = t.b, c = t.c, p = t.p, q = t.q;
    const T grx = g11 * a * a + g22 * b * b + g33 * p * p + g12 * a * b + g13 * a * p + g23 * b * p;
    const T gry = g11 * b * b + g22 * c * c + g33 * q * q + g12 * b * c + g13 * b * q + g23 * c * q;
    const T rx2 = rx * rx * grx, ry2 = ry * ry * gry;
    T* o = G + fk * 5 * hw + pix;
    o[0] = rx * ((T)2 * g11 * a + g12 * b + g13 * p) - (T)2 * a * rx2;
    o[hw] = rx * ((T)2 * g22 * b + g12 * a + g23 * p) + ry * ((T)2 * g11 * b + g12 * c + g13 * q) -
            (T)2 * b * (rx2 + ry2);
    o[2 * hw] = ry * ((T)2 * g22 * c + g12 * b + g23 * q) - (T)2 * c * ry2;
    o[3 * hw] = rx * ((T)2 * g33 * p + g13 * a + g23 * b);
    o[4 * hw] = ry * ((T)2 * g33 * q + g13 * b + g23 * c);
}

// Transposed difference stencils: gathers G into g_f1 (+)= S/2 - D parts and
// g_f2 = S/2 + D parts.  With clamped neighbours, the x positions whose
// left neighbour is X are {X+1} and {0 if X == 0}; those whose right
// neighbour is X are {X-1} and {w-1 if X == w-1}.
template <typename T>
__global__ void kd_tensor_adj_gather(const T* __restrict__ G, int K, int h, int w, T hy, T hx, T* __restrict__ gf1,
                                     T* __restrict__ gf2, int accumulate_f1)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    if (X >= w) return;
    const int Y = blockIdx.y;
    const long long fk = blockIdx.z, hw = (long long)h * w, pix = (long long)Y * w + X;
    const T* ga = G + fk * 5 * hw;
    const T* gb = ga + hw;
    const T* gc = ga + 2 * hw;
    const T* gp = ga + 3 * hw;
    const T* gq = ga + 4 * hw;
    auto at = [&](const T* a, int yy, int xx) { return a[(long long)yy * w + xx]; };
    // sums over the preimages of X under x -> x-1 (clamped) and x -> x+1 (clamped)
    auto sm_x = [&](const T* a, int yy, int xx) {
        return (xx + 1 <= w - 1 ? at(a, yy, xx + 1) : (T)0) + (xx == 0 ? at(a, yy, 0) : (T)0);
    };
    auto sp_x = [&](const T* a, int yy, int xx) {
        return (xx >= 1 ? at(a, yy, xx - 1) : (T)0) + (xx == w - 1 ? at(a, yy, w - 1) : (T)0);
    };
    auto sm_y = [&](const T* a, int yy, int xx) {
        return (yy + 1 <= h - 1 ? at(a, yy + 1, xx) : (T)0) + (yy == 0 ? at(a, 0, xx) : (T)0);
    };
    auto sp_y = [&](const T* a, int yy, int xx) {
        return (yy >= 1 ? at(a, yy - 1, xx) : (T)0) + (yy == h - 1 ? at(a, h - 1, xx) : (T)0);
    };
    const T i2hy = (T)1 / ((T)2 * hy), i2hx = (T)1 / ((T)2 * hx);
    auto gFX = [&](int r, int xx) { return (sp_y(gb, r, xx) - sm_y(gb, r, xx)) * i2hy; };
    // sums of gFX over the x-preimages of X
    T fx_p = (X >= 1 ? gFX(Y, X - 1) : (T)0) + (X == w - 1 ? gFX(Y, w - 1) : (T)0);
    T fx_m = (X + 1 <= w - 1 ? gFX(Y, X + 1) : (T)0) + (X == 0 ? gFX(Y, 0) : (T)0);
    const T gS = (sm_x(ga, Y, X) - (T)2 * at(ga, Y, X) + sp_x(ga, Y, X)) / (hx * hx) +
                 (sm_y(gc, Y, X) - (T)2 * at(gc, Y, X) + sp_y(gc, Y, X)) / (hy * hy) + (fx_p - fx_m) * i2hx;
    const T gD = (sp_x(gp, Y, X) - sm_x(gp, Y, X)) * i2hx + (sp_y(gq, Y, X) - sm_y(gq, Y, X)) * i2hy;
    const long long o = fk * hw + pix;
    const T g1 = (T)0.5 * gS - gD;
    gf1[o] = accumulate_f1 ? gf1[o] + g1 : g1;
    gf2[o] = (T)0.5 * gS + gD;
}

// ------------------------------------------------------------------ level solver
struct AData {
    double a[kMaxK];
};

// Coefficients per pixel (F, 5, h, w): max(A11, eps), max(A22, eps), A12,
// B1e, B2e, with A.. = sum_k W_k psi_k J.._k and the level's input flow folded
// into the constant terms, B1e = sum_k W psi J13 - ax lapx(u) - ay lapy(u)
// (lapx(u) = (u_L - u_c) + (u_R - u_c), clamped neighbours contributing 0),
// so that the sweeps read neither u nor v:
//   nu = -(B1e + A12 dv_c) + ax (du_L + du_R) + ay (du_T + du_B)
// which is the reference's -sum_k W psi (J13 + J12 dv) + sum_n w_n (u_n + du_n - u_c).

// Sums (va, vb) over the block and adds them to slot[0], slot[1], a pair
// owned by this block (no atomics: launches on one stream run in order and no
// other block of a launch writes the slot).  Every thread of the block calls it.
template <typename T>
__device__ __forceinline__ void block_add2(T va, T vb, double* slot)
{
    for (int o = 16; o > 0; o >>= 1) {
        va += __shfl_down_sync(0xffffffffu, va, o);
        vb += __shfl_down_sync(0xffffffffu, vb, o);
    }
    __shared__ T part[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        part[0][wid] = va;
        part[1][wid] = vb;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        va = lane < nw ? part[0][lane] : (T)0;
        vb = lane < nw ? part[1][lane] : (T)0;
        for (int o = 16; o > 0; o >>= 1) {
            va += __shfl_down_sync(0xffffffffu, va, o);
            vb += __shfl_down_sync(0xffffffffu, vb, o);
        }
        if (lane == 0) {
            slot[0] += (double)va;
            slot[1] += (double)vb;
        }
    }
    __syncthreads();
}

// The slot of this block in a per-launch-shape partial buffer: one pair per
// (frame, row, block column).
__device__ __forceinline__ double* block_slot(double* part)
{
    return part + ((((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x) + blockIdx.x) * 2;
}

// galpha(f, :) += sum of frame f's n_slots pairs, which are then cleared.
__global__ void kd_reduce_slots(double* __restrict__ part, long long n_slots, double* __restrict__ galpha)
{
    const long long f = blockIdx.x;
    double* p = part + f * n_slots * 2;
    double a = 0, b = 0;
    for (long long i = threadIdx.x; i < n_slots; i += blockDim.x) {
        a += p[2 * i];
        b += p[2 * i + 1];
        p[2 * i] = 0;
        p[2 * i + 1] = 0;
    }
    __shared__ double ra[256], rb[256];
    ra[threadIdx.x] = a;
    rb[threadIdx.x] = b;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            ra[threadIdx.x] += ra[threadIdx.x + st];
            rb[threadIdx.x] += rb[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        galpha[2 * f] += ra[0];
        galpha[2 * f + 1] += rb[0];
    }
}

// Solver state before a half-sweep: the values of each colour either from a
// compressed array of that colour's pixels (F, 2, h, (w + 1) / 2; pixel (y, x)
// at column x >> 1) or from a full array (F, 2, h, w); full == nullptr is zero.
template <typename T>
struct StateSrc {
    const T* full;
    const T* comp0;
    const T* comp1;
};

template <typename T>
__device__ __forceinline__ T sval(const StateSrc<T>& s, long long f, int plane, int y, int x, int h, int w, int hw2)
{
    const T* cp = ((x + y) & 1) ? s.comp1 : s.comp0;
    if (cp) return cp[((f * 2 + plane) * h + y) * (long long)hw2 + (x >> 1)];
    return s.full ? s.full[((f * 2 + plane) * h + y) * (long long)w + x] : (T)0;
}

// psi tick (torch/core/level_solver.py:73-117 with a_smooth = 1).  st: the
// full state (nullptr: zero); ck, when given, receives a copy of it.
template <typename T>
__global__ void kd_tick(const T* __restrict__ J, const T* __restrict__ W, const T* __restrict__ st,
                        const T* __restrict__ uv, int K, int h, int w, AData ad, T eps, T ax, T ay,
                        T* __restrict__ coef, T* __restrict__ ck)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long f = blockIdx.z, hw = (long long)h * w, pix = (long long)y * w + x;
    const T du = st ? st[f * 2 * hw + pix] : (T)0;
    const T dv = st ? st[f * 2 * hw + hw + pix] : (T)0;
    if (ck) {
        ck[f * 2 * hw + pix] = du;
        ck[f * 2 * hw + hw + pix] = dv;
    }
    const T* Jf = J + f * 6 * K * hw + pix;
    const long long qs = (long long)K * hw;
    T A11 = 0, A22 = 0, A12 = 0, B1 = 0, B2 = 0;
    for (int k = 0; k < K; ++k) {
        const T* j = Jf + k * hw;
        const T j11 = j[0], j22 = j[qs], j33 = j[2 * qs], j12 = j[3 * qs], j13 = j[4 * qs], j23 = j[5 * qs];
        T E = j11 * (du * du) + j22 * (dv * dv) + (T)2 * j12 * (du * dv) + (T)2 * j13 * du + (T)2 * j23 * dv + j33;
        E = E < (T)0 ? (T)0 : E;
        const T a = (T)ad.a[k];
        const T wpsi = W[k * hw + pix] * (a * tpow(E + eps, a - (T)1));
        A11 += wpsi * j11;
        A22 += wpsi * j22;
        A12 += wpsi * j12;
        B1 += wpsi * j13;
        B2 += wpsi * j23;
    }
    const T* u = uv + f * 2 * hw;
    const T* v = u + hw;
    const long long pL = x > 0 ? pix - 1 : pix, pR = x < w - 1 ? pix + 1 : pix;
    const long long pT = y > 0 ? pix - w : pix, pB = y < h - 1 ? pix + w : pix;
    const T lxu = (u[pL] - u[pix]) + (u[pR] - u[pix]), lyu = (u[pT] - u[pix]) + (u[pB] - u[pix]);
    const T lxv = (v[pL] - v[pix]) + (v[pR] - v[pix]), lyv = (v[pT] - v[pix]) + (v[pB] - v[pix]);
    T* c = coef + f * 5 * hw + pix;
    c[0] = tmax(A11, eps);
    c[hw] = tmax(A22, eps);
    c[2 * hw] = A12;
    c[3 * hw] = B1 - ax * lxu - ay * lyu;
    c[4 * hw] = B2 - ax * lxv - ay * lyv;
}

// One red-black half-sweep in place (torch/core/level_solver.py:119-199):
// pixels with (y + x) % 2 == color move.  gs = 0: du and dv of a moving pixel
// both from the state before the half-sweep (the torch backend); gs = 1: dv
// from the new du (the numba solver's within-pixel order,
// core/level_solver.py:355-364), which makes the sweep an SOR sweep of the
// symmetric positive definite system and keeps it convergent for omega < 2.
// store, when given, receives the moved pixels (compressed layout).  rhs,
// when given (F, 2, h, w), replaces (B1e, B2e) by (-rhs_u, -rhs_v): the same
// sweep then solves M lam = rhs for the level's symmetric operator M.
template <typename T>
__global__ void kd_rb_sweep(int color, const T* __restrict__ coef, const T* __restrict__ rhs, T* st,
                            T* __restrict__ store, int h, int w, T ax, T ay, T omega, T eps, int gs)
{
    const int tx = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int x = 2 * tx + ((y + color) & 1);
    if (x >= w) return;
    const long long f = blockIdx.z, hw = (long long)h * w, pc = (long long)y * w + x;
    T* du = st + f * 2 * hw;
    T* dv = du + hw;
    const long long pL = x > 0 ? pc - 1 : pc, pR = x < w - 1 ? pc + 1 : pc;
    const long long pT = y > 0 ? pc - w : pc, pB = y < h - 1 ? pc + w : pc;
    const T* c = coef + f * 5 * hw + pc;
    const T A11 = c[0], A22 = c[hw], A12 = c[2 * hw];
    const T B1 = rhs ? -rhs[f * 2 * hw + pc] : c[3 * hw], B2 = rhs ? -rhs[f * 2 * hw + hw + pc] : c[4 * hw];
    const T duc = du[pc], dvc = dv[pc];
    const T sw = ax + ax + ay + ay;
    const T nu = -(B1 + A12 * dvc) + ax * (du[pL] + du[pR]) + ay * (du[pT] + du[pB]);
    const T dun = ((T)1 - omega) * duc + omega * (nu / tmax(A11 + sw, eps));
    const T nv = -(B2 + A12 * (gs ? dun : duc)) + ax * (dv[pL] + dv[pR]) + ay * (dv[pT] + dv[pB]);
    const T dvn = ((T)1 - omega) * dvc + omega * (nv / tmax(A22 + sw, eps));
    du[pc] = dun;
    dv[pc] = dvn;
    if (store) {
        const int hw2 = (w + 1) >> 1;
        store[((f * 2) * h + y) * (long long)hw2 + tx] = dun;
        store[((f * 2 + 1) * h + y) * (long long)hw2 + tx] = dvn;
    }
}

// Adjoint of the half-sweeps of one window, in reverse, one kernel per
// half-sweep j over the pixels that move in it (colour c = j & 1).  lam is
// dL/d(state) (full layout, updated in place).  A pixel that does not move in
// half-sweep j + 1 only passes its gradient through and gathers
// w * a_{j+1} from its four moving neighbours; that gather is done here, just
// before the pixel's own step j (aprev: compressed a of step j + 1, or NULL
// for the window's last half-sweep).  Then, with av = omega * lam_v / den_v,
// lam_u' = lam_u - gs * A12 * av (with gs, dv read the new du) and
// au = omega * lam_u' / den_u, the step writes the pixel's new lam, its
// (au, av) to anext (read by the next, lower step and the closing gather),
// accumulates the coefficient gradients (gcoef: A11c, A22c, A12, B1e, B2e)
// and the (sx, sy)-scaled gradients of ax, ay into galpha (F, 2).
template <typename T>
__global__ void kd_rb_adj_step(int color, const T* __restrict__ coef, StateSrc<T> pre, T* __restrict__ lam,
                               const T* __restrict__ aprev, T* __restrict__ anext, int h, int w, T ax, T ay, T omega,
                               T eps, int gs, T* __restrict__ gcoef, double sx, double sy, double* __restrict__ galpha)
{
    const int tx = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long f = blockIdx.z, hw = (long long)h * w;
    const int hw2 = (w + 1) >> 1;
    const int x = 2 * tx + ((y + color) & 1);
    T gax = 0, gay = 0;
    if (x < w) {
        const long long pc = (long long)y * w + x;
        const bool hasL = x > 0, hasR = x < w - 1, hasT = y > 0, hasB = y < h - 1;
        T* lu = lam + f * 2 * hw;
        T* lv = lu + hw;
        T lamu = lu[pc], lamv = lv[pc];
        if (aprev) {
            // neighbours have the other colour: compressed column x >> 1 of their row
            const T* apu = aprev + (f * 2 * h) * (long long)hw2;
            const T* apv = apu + (long long)h * hw2;
            T su = 0, sv = 0;
            if (hasL) { const long long q = (long long)y * hw2 + ((x - 1) >> 1); su += ax * apu[q]; sv += ax * apv[q]; }
            if (hasR) { const long long q = (long long)y * hw2 + ((x + 1) >> 1); su += ax * apu[q]; sv += ax * apv[q]; }
            if (hasT) { const long long q = (long long)(y - 1) * hw2 + (x >> 1); su += ay * apu[q]; sv += ay * apv[q]; }
            if (hasB) { const long long q = (long long)(y + 1) * hw2 + (x >> 1); su += ay * apu[q]; sv += ay * apv[q]; }
            lamu += su;
            lamv += sv;
        }
        const T* cf = coef + f * 5 * hw + pc;
        const T A12 = cf[2 * hw], B1 = cf[3 * hw], B2 = cf[4 * hw];
        const T sw = ax + ax + ay + ay;
        const T idu = (T)1 / tmax(cf[0] + sw, eps), idv = (T)1 / tmax(cf[hw] + sw, eps);
        const T av = omega * lamv * idv;
        const T lue = gs ? lamu - A12 * av : lamu;
        const T au = omega * lue * idu;
        const int xl = hasL ? x - 1 : x, xr = hasR ? x + 1 : x, yt = hasT ? y - 1 : y, yb = hasB ? y + 1 : y;
        const T duc = sval(pre, f, 0, y, x, h, w, hw2), dvc = sval(pre, f, 1, y, x, h, w, hw2);
        const T Xdu = sval(pre, f, 0, y, xl, h, w, hw2) + sval(pre, f, 0, y, xr, h, w, hw2);
        const T Ydu = sval(pre, f, 0, yt, x, h, w, hw2) + sval(pre, f, 0, yb, x, h, w, hw2);
        const T Xdv = sval(pre, f, 1, y, xl, h, w, hw2) + sval(pre, f, 1, y, xr, h, w, hw2);
        const T Ydv = sval(pre, f, 1, yt, x, h, w, hw2) + sval(pre, f, 1, yb, x, h, w, hw2);
        const T ru = (-(B1 + A12 * dvc) + ax * Xdu + ay * Ydu) * idu;
        const T dun = ((T)1 - omega) * duc + omega * ru;
        const T du_for_v = gs ? dun : duc;
        const T rv = (-(B2 + A12 * du_for_v) + ax * Xdv + ay * Ydv) * idv;
        // border reflections of this pixel read its own du / dv
        const T self = ax * (T)((hasL ? 0 : 1) + (hasR ? 0 : 1)) + ay * (T)((hasT ? 0 : 1) + (hasB ? 0 : 1));
        lu[pc] = ((T)1 - omega) * lue + self * au - (gs ? (T)0 : A12 * av);
        lv[pc] = ((T)1 - omega) * lamv - A12 * au + self * av;
        T* an = anext + (f * 2 * h + y) * (long long)hw2 + tx;
        an[0] = au;
        an[(long long)h * hw2] = av;
        T* g = gcoef + f * 5 * hw + pc;
        g[0] -= au * ru;
        g[hw] -= av * rv;
        g[2 * hw] -= au * dvc + av * du_for_v;
        g[3 * hw] -= au;
        g[4 * hw] -= av;
        const T rr = (T)2 * (au * ru + av * rv);
        gax = (au * Xdu + av * Xdv - rr) * (T)sx;
        gay = (au * Ydu + av * Ydv - rr) * (T)sy;
    }
    block_add2(gax, gay, block_slot(galpha));
}

// Asynchronous copy of one element global -> shared (cp.async, 4 or 8 bytes).
template <typename T>
__device__ __forceinline__ void cp_async_el(T* dst, const T* src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Two-element vector of T (float2 / double2) for the paired shared-memory planes.
template <typename T>
struct Vec2T;
template <>
struct Vec2T<float> {
    using type = float2;
};
template <>
struct Vec2T<double> {
    using type = double2;
};

// Solver state of one colour before a half-sweep, as kd_rb_adj_window stages
// it: kind 0 zero, 1 a full array (F, 2, h, w), 2 a compressed array of that
// colour's pixels (F, 2, h, (w + 1) / 2).
template <typename T>
struct StateSlice {
    const T* p;
    int kind;
};

// Copies colour c of a state slice over the window's outer region (origin
// (rx1, ry1), Rh1 rows of Rp1 pixel pairs; pair k of a row holds columns
// rx1 + 2k and rx1 + 2k + 1, one of each colour) into dst, one (du, dv) pair
// per entry row * Rp1 + k.  Pixels outside the level are left alone (never
// read).  Issues cp.async copies and commits them.
template <typename T>
__device__ __forceinline__ void stage_colour(typename Vec2T<T>::type* dst, int c, StateSlice<T> src, long long f,
                                             int h, int w, int hw2, int rx1, int ry1, int Rh1, int Rp1, float inv_rp1)
{
    const int n = Rh1 * Rp1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int row = (int)(((float)i + 0.5f) * inv_rp1);
        const int k = i - row * Rp1;
        const int gy = ry1 + row;
        const int gx = rx1 + 2 * k + ((c - rx1 - gy) & 1);
        if (gy < 0 || gy >= h || gx < 0 || gx >= w) continue;
        T* d = reinterpret_cast<T*>(dst + i);
        if (src.kind == 0) {
            d[0] = (T)0;
            d[1] = (T)0;
        } else if (src.kind == 1) {
            const T* q = src.p + ((f * 2) * h + gy) * (long long)w + gx;
            cp_async_el(d, q);
            cp_async_el(d + 1, q + (long long)h * w);
        } else {
            const T* q = src.p + ((f * 2) * h + gy) * (long long)hw2 + (gx >> 1);
            cp_async_el(d, q);
            cp_async_el(d + 1, q + (long long)h * hw2);
        }
    }
    cp_async_commit();
}

// Shared-memory planes of kd_rb_adj_window over the tile grown by nh: C0 =
// (A12, B1e), C1 = (B2e, 1 / den_u), C2 = 1 / den_v, L = lam, A = the latest
// (au, av).
template <typename T>
struct AdjPlanes {
    typename Vec2T<T>::type *C0, *C1, *L, *A;
    T* C2;
};

// One pixel's step of kd_rb_adj_window: the arithmetic of kd_rb_adj_step on
// the shared-memory planes.  Entry e of a ring table gives li (the pixel in
// the planes, row pitch Rw), sb (its pair in the staged states, row pitch Rp1)
// and p (its column parity in the pair): its own state is in `own`, its
// neighbours' (the other colour) in `oth`.  EDGE: the tile's outer region
// reaches the level's border, so neighbours may be missing (the pixel's own
// value stands in for them, as the border copies of the reference do);
// without EDGE every neighbour exists.  In two parts, load and step, so that
// a thread can load two pixels before it computes either.
template <typename T>
struct AdjPx {
    typename Vec2T<T>::type lam, c0, c1, st;
    T idv, Xdu, Ydu, Xdv, Ydv, self;
    int li;
};

template <typename T, bool EDGE>
__device__ __forceinline__ void adj_px_load(AdjPx<T>& q, int2 e, int x0, int y0, int h, int w, int Rw, int Rp1,
                                            bool gather, const typename Vec2T<T>::type* own,
                                            const typename Vec2T<T>::type* oth, T ax, T ay, const AdjPlanes<T>& P)
{
    using V2 = typename Vec2T<T>::type;
    const int li = e.y & 0x1fff, sb = (e.y >> 13) & 0x1fff, p = (e.y >> 26) & 1;
    bool hasL = true, hasR = true, hasT = true, hasB = true;
    if (EDGE) {
        const int gx = x0 + (int)(short)(e.x & 0xffff), gy = y0 + (e.x >> 16);
        hasL = gx > 0;
        hasR = gx < w - 1;
        hasT = gy > 0;
        hasB = gy < h - 1;
    }
    q.li = li;
    q.lam = P.L[li];
    if (gather) {
        T su = 0, sv = 0;
        if (hasL) { const V2 a = P.A[li - 1]; su += ax * a.x; sv += ax * a.y; }
        if (hasR) { const V2 a = P.A[li + 1]; su += ax * a.x; sv += ax * a.y; }
        if (hasT) { const V2 a = P.A[li - Rw]; su += ay * a.x; sv += ay * a.y; }
        if (hasB) { const V2 a = P.A[li + Rw]; su += ay * a.x; sv += ay * a.y; }
        q.lam.x += su;
        q.lam.y += sv;
    }
    q.c0 = P.C0[li];
    q.c1 = P.C1[li];
    q.idv = P.C2[li];
    q.st = own[sb];
    const V2 sl = hasL ? oth[sb - 1 + p] : q.st, sr = hasR ? oth[sb + p] : q.st;
    const V2 st_ = hasT ? oth[sb - Rp1] : q.st, sbm = hasB ? oth[sb + Rp1] : q.st;
    q.Xdu = sl.x + sr.x;
    q.Ydu = st_.x + sbm.x;
    q.Xdv = sl.y + sr.y;
    q.Ydv = st_.y + sbm.y;
    q.self = EDGE ? ax * (T)((hasL ? 0 : 1) + (hasR ? 0 : 1)) + ay * (T)((hasT ? 0 : 1) + (hasB ? 0 : 1)) : (T)0;
}

// The step itself; with ACC the coefficient gradients go to g and the
// (sx, sy)-scaled alpha gradients to (gax, gay).  Writes lam and (au, av).
template <typename T, bool ACC>
__device__ __forceinline__ void adj_px_step(const AdjPx<T>& q, T ax, T ay, T omega, int gs, const AdjPlanes<T>& P,
                                            T (&g)[5], T& gax, T& gay, T sx, T sy)
{
    using V2 = typename Vec2T<T>::type;
    const T A12 = q.c0.x, B1 = q.c0.y, B2 = q.c1.x, idu = q.c1.y, idv = q.idv;
    const T duc = q.st.x, dvc = q.st.y;
    const T av = omega * q.lam.y * idv;
    const T lue = gs ? q.lam.x - A12 * av : q.lam.x;
    const T au = omega * lue * idu;
    const T ru = (-(B1 + A12 * dvc) + ax * q.Xdu + ay * q.Ydu) * idu;
    const T dun = ((T)1 - omega) * duc + omega * ru;
    const T du_for_v = gs ? dun : duc;
    const T rv = (-(B2 + A12 * du_for_v) + ax * q.Xdv + ay * q.Ydv) * idv;
    V2 nl;
    nl.x = ((T)1 - omega) * lue + q.self * au - (gs ? (T)0 : A12 * av);
    nl.y = ((T)1 - omega) * q.lam.y - A12 * au + q.self * av;
    P.L[q.li] = nl;
    V2 na;
    na.x = au;
    na.y = av;
    P.A[q.li] = na;
    if (ACC) {
        g[0] -= au * ru;
        g[1] -= av * rv;
        g[2] -= au * dvc + av * du_for_v;
        g[3] -= au;
        g[4] -= av;
        const T rr = (T)2 * (au * ru + av * rv);
        gax += (au * q.Xdu + av * q.Xdv - rr) * sx;
        gay += (au * q.Ydu + av * q.Ydv - rr) * sy;
    }
}

// The steps of one window, from half-sweep nh - 1 down to 0 (see
// kd_rb_adj_window).
template <typename T, bool EDGE>
__device__ __forceinline__ void adj_window_steps(int nh, int x0, int y0, int h, int w, int Rw, int Rp1, int n1,
                                                 int nin, const int2* sTab, int nt0, const AdjTable& tab,
                                                 typename Vec2T<T>::type* sS, const T* s0, const T* hist, long long slot, long long f, int hw2,
                                                 int rx1, int ry1, int Rh1, float inv_rp1, T ax, T ay, T omega,
                                                 int gs, const AdjPlanes<T>& PL, T (&g0)[5], T (&g1)[5], T& gax,
                                                 T& gay, T tsx, T tsy)
{
    using V2 = typename Vec2T<T>::type;
    T dummy[5];
    T dax = 0, day = 0;
    auto slice = [&](int k) -> StateSlice<T> {
        if (k >= 0) return StateSlice<T>{hist + (long long)k * slot, 2};
        return StateSlice<T>{s0, s0 ? 1 : 0};
    };
    auto buf = [&](int c, int b) { return sS + (c * 2 + b) * n1; };
    int cur[2] = {0, 0};
    for (int j = nh - 1; j >= 0; --j) {
        const int c = j & 1;
        const V2* own = buf(c, cur[c]);
        const V2* oth = buf(c ^ 1, cur[c ^ 1]);
        // the other colour's state for step j - 1 (its values after j - 3), one step ahead
        if (j >= 1)
            stage_colour<T>(buf(c ^ 1, cur[c ^ 1] ^ 1), c ^ 1, slice(j - 3), f, h, w, hw2, rx1, ry1, Rh1, Rp1,
                            inv_rp1);
        const bool gather = j < nh - 1;
        // the moving pixels within j + 1 of the tile: the first cnt entries of this colour's ring table;
        // entry t is this thread's own tile pixel, the others (halo) come two at a time, both loaded
        // before either is computed (pixels of one colour do not read each other)
        const int2* te = sTab + (c ? nt0 : 0);
        const int n_act = tab.cnt[c][j + 1];
        const int bd = blockDim.x;
        auto inside = [&](int2 e) {
            if (!EDGE) return true;
            const int gx = x0 + (int)(short)(e.x & 0xffff), gy = y0 + (e.x >> 16);
            return gx >= 0 && gy >= 0 && gx < w && gy < h;
        };
        {
            const int2 e = te[threadIdx.x];
            if (inside(e)) {
                AdjPx<T> q;
                adj_px_load<T, EDGE>(q, e, x0, y0, h, w, Rw, Rp1, gather, own, oth, ax, ay, PL);
                if (c == 0)
                    adj_px_step<T, true>(q, ax, ay, omega, gs, PL, g0, gax, gay, tsx, tsy);
                else
                    adj_px_step<T, true>(q, ax, ay, omega, gs, PL, g1, gax, gay, tsx, tsy);
            }
        }
        for (int i = nin + threadIdx.x; i < n_act; i += 2 * bd) {
            const int2 ea = te[i];
            const bool ha = inside(ea);
            const bool hb = i + bd < n_act && inside(te[i + bd]);
            AdjPx<T> qa, qb;
            if (ha) adj_px_load<T, EDGE>(qa, ea, x0, y0, h, w, Rw, Rp1, gather, own, oth, ax, ay, PL);
            if (hb) adj_px_load<T, EDGE>(qb, te[i + bd], x0, y0, h, w, Rw, Rp1, gather, own, oth, ax, ay, PL);
            if (ha) adj_px_step<T, false>(qa, ax, ay, omega, gs, PL, dummy, dax, day, tsx, tsy);
            if (hb) adj_px_step<T, false>(qb, ax, ay, omega, gs, PL, dummy, dax, day, tsx, tsy);
        }
        cp_async_wait_all();
        __syncthreads();
        cur[c ^ 1] ^= 1;
    }
}

// Adjoint of all nh half-sweeps of one tick window in one launch (temporal
// blocking), with kd_rb_adj_step's arithmetic.  A CTA owns a TX x TY tile of
// one frame (TX = TY = 16 or 32) and keeps in shared memory:
//  * over the tile grown by nh pixels on every side (Rw x Rh): (A12, B1e),
//    (B2e, 1 / den_u), 1 / den_v, lam and the pixel's latest (au, av);
//  * over the tile grown by nh + 1 (Rh1 rows of Rp1 pixel pairs), per colour
//    two buffers of the solver state (du, dv) before a half-sweep, filled by
//    cp.async from the window's stored half-sweeps (hist + j * slot,
//    compressed; s0, NULL: zero, before the first) one step ahead: before
//    half-sweep j the moving colour holds its values after j - 2 and the other
//    colour after j - 1, so each step replaces one colour;
//  * the two colours' ring tables (AdjTable).
// lam of the tile after the window depends on the pixels within j + 1 of the
// tile at half-sweep j, so step j (from nh - 1 down to 0) updates the moving
// pixels of that shrinking region: the tile's own pixels and a halo that
// neighbouring tiles also compute.  They come from the ring table of the
// step's colour (the tile first, entry t the pixel of thread t's horizontal
// pair, then the rings at distance 1, 2, ...), so a step's pixels are its
// first cnt[c][j + 1] entries and the threads stay busy as the region shrinks.
// Thread t keeps its pair's coefficient gradients and its alpha gradients in
// registers for the whole window.  Tiles whose outer region lies inside the
// level take a path without border tests.  The window ends with the closing
// gather of the tile's colour-1 pixels (kd_rb_adj_gather); the tile's lam goes
// to lam_out, which is not lam_in (tiles read each other's halo), and its
// coefficient gradients overwrite gcoef.  blockDim.x = TX * TY / 2.
template <typename T>
__global__ void __launch_bounds__(512) kd_rb_adj_window(const T* __restrict__ coef, const T* __restrict__ s0,
                                                         const T* __restrict__ hist, long long slot,
                                                         const T* __restrict__ lam_in, T* __restrict__ lam_out, int h,
                                                         int w, int nh, int TX, int TY, AdjTable tab, T ax, T ay,
                                                         T omega, T eps, int gs, T* __restrict__ gcoef, double sx,
                                                         double sy, double* __restrict__ galpha)
{
    using V2 = typename Vec2T<T>::type;
    extern __shared__ __align__(16) unsigned char smraw[];
    T* const sm = reinterpret_cast<T*>(smraw);
    const int Rw = TX + 2 * nh, Rh = TY + 2 * nh, R = Rw * Rh;
    const int Rp1 = (Rw + 2) >> 1, Rh1 = Rh + 2, n1 = Rh1 * Rp1;
    // R is even (TX even), so every V2 plane starts on a V2 boundary
    AdjPlanes<T> PL;
    PL.C0 = reinterpret_cast<V2*>(sm);
    PL.C1 = reinterpret_cast<V2*>(sm + 2 * R);
    PL.C2 = sm + 4 * R;
    PL.L = reinterpret_cast<V2*>(sm + 5 * R);
    PL.A = reinterpret_cast<V2*>(sm + 7 * R);
    V2* const sS = reinterpret_cast<V2*>(sm + 9 * R);  // state buffers: (colour * 2 + buffer) * n1
    int2* const sTab = reinterpret_cast<int2*>(sS + 4 * n1);
    const int nt0 = tab.cnt[0][nh], nt1 = tab.cnt[1][nh];
    for (int i = threadIdx.x; i < nt0; i += blockDim.x) sTab[i] = tab.e[0][i];
    for (int i = threadIdx.x; i < nt1; i += blockDim.x) sTab[nt0 + i] = tab.e[1][i];
    const long long f = blockIdx.z, hw = (long long)h * w;
    const int hw2 = (w + 1) >> 1;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int rx0 = x0 - nh, ry0 = y0 - nh;
    const int rx1 = rx0 - 1, ry1 = ry0 - 1;
    const float inv_rp1 = 1.0f / (float)Rp1;
    auto slice = [&](int k) -> StateSlice<T> {
        if (k >= 0) return StateSlice<T>{hist + (long long)k * slot, 2};
        return StateSlice<T>{s0, s0 ? 1 : 0};
    };
    // the states before the window's last half-sweep nh - 1 (colour 1): colour 1
    // after nh - 3 into its buffer 0, colour 0 after nh - 2 into its buffer 0
    stage_colour<T>(sS + 2 * n1, 1, slice(nh - 3), f, h, w, hw2, rx1, ry1, Rh1, Rp1, inv_rp1);
    stage_colour<T>(sS, 0, slice(nh - 2), f, h, w, hw2, rx1, ry1, Rh1, Rp1, inv_rp1);
    // the coefficients and lam over the tile grown by nh, copied asynchronously (the two
    // denominators raw, turned into reciprocals once they have arrived)
    const float inv_rw = 1.0f / (float)Rw;
    {
        const T* cf = coef + f * 5 * hw;
        const T* liu = lam_in + f * 2 * hw;
        const T* liv = liu + hw;
        for (int i = threadIdx.x; i < R; i += blockDim.x) {
            const int ry = (int)(((float)i + 0.5f) * inv_rw);
            const int gy = ry0 + ry, gx = rx0 + (i - ry * Rw);
            if (gy >= 0 && gy < h && gx >= 0 && gx < w) {
                const long long q = (long long)gy * w + gx;
                T* c0 = reinterpret_cast<T*>(PL.C0 + i);
                T* c1 = reinterpret_cast<T*>(PL.C1 + i);
                T* l = reinterpret_cast<T*>(PL.L + i);
                cp_async_el(c0, cf + 2 * hw + q);
                cp_async_el(c0 + 1, cf + 3 * hw + q);
                cp_async_el(c1, cf + 4 * hw + q);
                cp_async_el(c1 + 1, cf + q);
                cp_async_el(PL.C2 + i, cf + hw + q);
                cp_async_el(l, liu + q);
                cp_async_el(l + 1, liv + q);
            }
        }
        cp_async_commit();
    }
    cp_async_wait_all();
    __syncthreads();
    {
        const T sw = ax + ax + ay + ay;
        for (int i = threadIdx.x; i < R; i += blockDim.x) {
            const int ry = (int)(((float)i + 0.5f) * inv_rw);
            const int gy = ry0 + ry, gx = rx0 + (i - ry * Rw);
            if (gy >= 0 && gy < h && gx >= 0 && gx < w) {
                PL.C1[i].y = (T)1 / tmax(PL.C1[i].y + sw, eps);
                PL.C2[i] = (T)1 / tmax(PL.C2[i] + sw, eps);
            }
        }
    }
    __syncthreads();
    T g0[5] = {0, 0, 0, 0, 0}, g1[5] = {0, 0, 0, 0, 0};  // the thread's colour-0 and colour-1 pixels
    T gax = 0, gay = 0;
    const T tsx = (T)sx, tsy = (T)sy;
    const int nin = (TX * TY) >> 1;  // entries 0 .. nin - 1 of a colour: the tile's own pixels, thread t's at t
    const bool edge = rx1 < 0 || ry1 < 0 || rx1 + 2 * Rp1 > w || ry1 + Rh1 > h;
    if (edge)
        adj_window_steps<T, true>(nh, x0, y0, h, w, Rw, Rp1, n1, nin, sTab, nt0, tab, sS, s0, hist, slot, f,
                                  hw2, rx1, ry1, Rh1, inv_rp1, ax, ay, omega, gs, PL, g0, g1, gax, gay, tsx, tsy);
    else
        adj_window_steps<T, false>(nh, x0, y0, h, w, Rw, Rp1, n1, nin, sTab, nt0, tab, sS, s0, hist, slot, f,
                                   hw2, rx1, ry1, Rh1, inv_rp1, ax, ay, omega, gs, PL, g0, g1, gax, gay, tsx, tsy);
    // the closing gather (colour 1), then the tile's lam and coefficient gradients
    T* lou = lam_out + f * 2 * hw;
    T* gc = gcoef + f * 5 * hw;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const int2 e = sTab[(c ? nt0 : 0) + threadIdx.x];
        const int px = x0 + (int)(short)(e.x & 0xffff), py = y0 + (e.x >> 16);
        if (py < h && px < w) {
            const int li = e.y & 0x1fff;
            V2 l = PL.L[li];
            if (c == 1) {
                T su = 0, sv = 0;
                if (px > 0) { const V2 a = PL.A[li - 1]; su += ax * a.x; sv += ax * a.y; }
                if (px < w - 1) { const V2 a = PL.A[li + 1]; su += ax * a.x; sv += ax * a.y; }
                if (py > 0) { const V2 a = PL.A[li - Rw]; su += ay * a.x; sv += ay * a.y; }
                if (py < h - 1) { const V2 a = PL.A[li + Rw]; su += ay * a.x; sv += ay * a.y; }
                l.x += su;
                l.y += sv;
            }
            const long long q = (long long)py * w + px;
            lou[q] = l.x;
            lou[hw + q] = l.y;
            const T* gg = c == 0 ? g0 : g1;
#pragma unroll
            for (int k = 0; k < 5; ++k) gc[k * hw + q] = gg[k];
        }
    }
    block_add2(gax, gay, block_slot(galpha));
}

// The closing gather of a window: pixels of colour `color` (which did not move
// in the window's first half-sweep) add w * a_0 of their moving neighbours.
template <typename T>
__global__ void kd_rb_adj_gather(int color, T* __restrict__ lam, const T* __restrict__ aprev, int h, int w, T ax,
                                 T ay)
{
    const int tx = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int x = 2 * tx + ((y + color) & 1);
    if (x >= w) return;
    const long long f = blockIdx.z, hw = (long long)h * w, pc = (long long)y * w + x;
    const int hw2 = (w + 1) >> 1;
    const T* apu = aprev + (f * 2 * h) * (long long)hw2;
    const T* apv = apu + (long long)h * hw2;
    T su = 0, sv = 0;
    if (x > 0) { const long long q = (long long)y * hw2 + ((x - 1) >> 1); su += ax * apu[q]; sv += ax * apv[q]; }
    if (x < w - 1) { const long long q = (long long)y * hw2 + ((x + 1) >> 1); su += ax * apu[q]; sv += ax * apv[q]; }
    if (y > 0) { const long long q = (long long)(y - 1) * hw2 + (x >> 1); su += ay * apu[q]; sv += ay * apv[q]; }
    if (y < h - 1) { const long long q = (long long)(y + 1) * hw2 + (x >> 1); su += ay * apu[q]; sv += ay * apv[q]; }
    lam[f * 2 * hw + pc] += su;
    lam[f * 2 * hw + hw + pc] += sv;
}

// Implicit adjoint of a level (psi held at its last tick): with the solver's
// fixed point M x = b, b = -(B1e, B2e), and lam = M^-1 dL/dx, the gradients
// are dL/db = lam and dL/dM = -lam x^T.  Per pixel this gives the coefficient
// gradients (gcoef, overwritten) and, through M's dependence on ax and ay
// (diagonal 2 ax + 2 ay, neighbours -ax / -ay, clamped neighbours reading the
// pixel itself), the (sx, sy)-scaled gradients of ax, ay into galpha.
template <typename T>
__global__ void kd_implicit_assemble(const T* __restrict__ lam, const T* __restrict__ x, int h, int w,
                                     T* __restrict__ gcoef, double sx, double sy, double* __restrict__ galpha)
{
    const int xx = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long f = blockIdx.z, hw = (long long)h * w;
    T gax = 0, gay = 0;
    if (xx < w) {
        const long long pc = (long long)y * w + xx;
        const T* du = x + f * 2 * hw;
        const T* dv = du + hw;
        const T lu = lam[f * 2 * hw + pc], lv = lam[f * 2 * hw + hw + pc];
        const long long pL = xx > 0 ? pc - 1 : pc, pR = xx < w - 1 ? pc + 1 : pc;
        const long long pT = y > 0 ? pc - w : pc, pB = y < h - 1 ? pc + w : pc;
        const T duc = du[pc], dvc = dv[pc];
        T* g = gcoef + f * 5 * hw + pc;
        g[0] = -lu * duc;
        g[hw] = -lv * dvc;
        g[2 * hw] = -(lu * dvc + lv * duc);
        g[3 * hw] = -lu;
        g[4 * hw] = -lv;
        gax = -(lu * ((T)2 * duc - du[pL] - du[pR]) + lv * ((T)2 * dvc - dv[pL] - dv[pR])) * (T)sx;
        gay = -(lu * ((T)2 * duc - du[pT] - du[pB]) + lv * ((T)2 * dvc - dv[pT] - dv[pB])) * (T)sy;
    }
    block_add2(gax, gay, block_slot(galpha));
}

// Adjoint of a psi tick and of the folded input flow, once per window:
// coefficient gradients -> g_J (accumulated); unless lagged, the gradient of
// the tick state through E into lam; the gradient of the level's input flow
// through B1e, B2e into guv; that of ax, ay into galpha.  lagged = 1 holds psi
// fixed (no derivative of psi with respect to the tick state or J33).
template <typename T, int KT>
__global__ void kd_tick_adj(const T* __restrict__ J, const T* __restrict__ W, const T* __restrict__ st,
                            const T* __restrict__ uv, const T* __restrict__ gcoef, int K_, int h, int w, AData ad,
                            T eps, T ax, T ay, int lagged, T* __restrict__ gJ, T* __restrict__ lam,
                            T* __restrict__ guv, double sx, double sy, double* __restrict__ galpha)
{
    // KT > 0: the channel count at compile time (psi and E stay in registers); 0: K_ at run time
    constexpr int KA = KT > 0 ? KT : kMaxK;
    const int K = KT > 0 ? KT : K_;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long f = blockIdx.z, hw = (long long)h * w;
    T gax = 0, gay = 0;
    if (x < w) {
        const long long pix = (long long)y * w + x;
        const T du = st ? st[f * 2 * hw + pix] : (T)0;
        const T dv = st ? st[f * 2 * hw + hw + pix] : (T)0;
        const T* Jf = J + f * 6 * K * hw + pix;
        T* gJf = gJ + f * 6 * K * hw + pix;
        const long long qs = (long long)K * hw;
        // with the channel count known, the accumulated tensor gradients are read up front, so
        // their loads overlap the power and the other loads instead of following them
        T gjp[KT > 0 ? 6 * KT : 1];
        if constexpr (KT > 0) {
#pragma unroll
            for (int k = 0; k < KT; ++k)
#pragma unroll
                for (int q = 0; q < 6; ++q) gjp[k * 6 + q] = gJf[k * hw + q * qs];
        }
        // psi and the raw sums (for the max(., eps) clamps), as kd_tick computes them
        T psi[KA], Er[KA];
        T A11 = 0, A22 = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const T* j = Jf + k * hw;
            Er[k] = j[0] * (du * du) + j[qs] * (dv * dv) + (T)2 * j[3 * qs] * (du * dv) + (T)2 * j[4 * qs] * du +
                    (T)2 * j[5 * qs] * dv + j[2 * qs];
            const T E = Er[k] < (T)0 ? (T)0 : Er[k];
            const T a = (T)ad.a[k];
            psi[k] = a * tpow(E + eps, a - (T)1);
            const T wpsi = W[k * hw + pix] * psi[k];
            A11 += wpsi * j[0];
            A22 += wpsi * j[qs];
        }
        const T* gc = gcoef + f * 5 * hw;
        // torch.maximum splits the gradient evenly on a tie
        const T g11 = gc[pix] * (A11 > eps ? (T)1 : (A11 == eps ? (T)0.5 : (T)0));
        const T g22 = gc[hw + pix] * (A22 > eps ? (T)1 : (A22 == eps ? (T)0.5 : (T)0));
        const T g12 = gc[2 * hw + pix], gb1 = gc[3 * hw + pix], gb2 = gc[4 * hw + pix];
        T ldu = 0, ldv = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const T* j = Jf + k * hw;
            T* gj = gJf + k * hw;
            const T j11 = j[0], j22 = j[qs], j12 = j[3 * qs], j13 = j[4 * qs], j23 = j[5 * qs];
            const T Wk = W[k * hw + pix];
            const T wpsi = Wk * psi[k];
            T g11k = g11 * wpsi, g22k = g22 * wpsi, g33k = 0, g12k = g12 * wpsi, g13k = gb1 * wpsi, g23k = gb2 * wpsi;
            if (!lagged && Er[k] >= (T)0) {
                // clamp_min passes the gradient where E >= 0; dpsi/dE = (a - 1) psi / (E + eps)
                const T E = Er[k];
                const T a = (T)ad.a[k];
                const T gpsi = Wk * (g11 * j11 + g22 * j22 + g12 * j12 + gb1 * j13 + gb2 * j23);
                const T gE = gpsi * ((a - (T)1) * psi[k] / (E + eps));
                g11k += gE * (du * du);
                g22k += gE * (dv * dv);
                g33k += gE;
                g12k += gE * (T)2 * (du * dv);
                g13k += gE * (T)2 * du;
                g23k += gE * (T)2 * dv;
                ldu += gE * ((T)2 * j11 * du + (T)2 * j12 * dv + (T)2 * j13);
                ldv += gE * ((T)2 * j22 * dv + (T)2 * j12 * du + (T)2 * j23);
            }
            if constexpr (KT > 0) {
                gj[0] = gjp[k * 6 + 0] + g11k;
                gj[qs] = gjp[k * 6 + 1] + g22k;
                gj[2 * qs] = gjp[k * 6 + 2] + g33k;
                gj[3 * qs] = gjp[k * 6 + 3] + g12k;
                gj[4 * qs] = gjp[k * 6 + 4] + g13k;
                gj[5 * qs] = gjp[k * 6 + 5] + g23k;
            } else {
                gj[0] += g11k;
                gj[qs] += g22k;
                gj[2 * qs] += g33k;
                gj[3 * qs] += g12k;
                gj[4 * qs] += g13k;
                gj[5 * qs] += g23k;
            }
        }
        if (lam && !lagged) {
            lam[f * 2 * hw + pix] += ldu;
            lam[f * 2 * hw + hw + pix] += ldv;
        }
        // B1e(p) = B1 - ax lapx(u)(p) - ay lapy(u)(p): gather over the pixels whose
        // Laplacian reads u at this pixel (its interior neighbours and itself)
        const bool hasL = x > 0, hasR = x < w - 1, hasT = y > 0, hasB = y < h - 1;
        const T nx = (T)((hasL ? 1 : 0) + (hasR ? 1 : 0)), ny = (T)((hasT ? 1 : 0) + (hasB ? 1 : 0));
        const T* g1 = gc + 3 * hw;
        const T* g2 = gc + 4 * hw;
        T sxb1 = 0, syb1 = 0, sxb2 = 0, syb2 = 0;
        if (hasL) { sxb1 += g1[pix - 1]; sxb2 += g2[pix - 1]; }
        if (hasR) { sxb1 += g1[pix + 1]; sxb2 += g2[pix + 1]; }
        if (hasT) { syb1 += g1[pix - w]; syb2 += g2[pix - w]; }
        if (hasB) { syb1 += g1[pix + w]; syb2 += g2[pix + w]; }
        T* gu = guv + f * 2 * hw;
        gu[pix] += -ax * sxb1 - ay * syb1 + (ax * nx + ay * ny) * gb1;
        gu[hw + pix] += -ax * sxb2 - ay * syb2 + (ax * nx + ay * ny) * gb2;
        const T* u = uv + f * 2 * hw;
        const T* v = u + hw;
        const long long pL = hasL ? pix - 1 : pix, pR = hasR ? pix + 1 : pix;
        const long long pT = hasT ? pix - w : pix, pB = hasB ? pix + w : pix;
        const T lxu = (u[pL] - u[pix]) + (u[pR] - u[pix]), lyu = (u[pT] - u[pix]) + (u[pB] - u[pix]);
        const T lxv = (v[pL] - v[pix]) + (v[pR] - v[pix]), lyv = (v[pT] - v[pix]) + (v[pB] - v[pix]);
        gax = -(gb1 * lxu + gb2 * lxv) * (T)sx;
        gay = -(gb1 * lyu + gb2 * lyv) * (T)sy;
    }
    block_add2(gax, gay, block_slot(galpha));
}

// ------------------------------------------------------------------ median
// 5x5 median with mirror borders (scipy.ndimage.median_filter(size=5,
// mode="mirror"), core/optical_flow.py:607-609): a bitonic sorting network
// over 32 slots (25 values, 7 of +inf) with compile-time indices, so the
// values stay in registers; each slot carries its source index, and the
// 13th smallest is returned with the index it came from.
template <typename T>
__device__ __forceinline__ void cswap(T& a, T& b, int& ia, int& ib, bool up)
{
    const bool sw = up ? (b < a) : (a < b);
    const T ta = sw ? b : a, tb = sw ? a : b;
    const int ja = sw ? ib : ia, jb = sw ? ia : ib;
    a = ta;
    b = tb;
    ia = ja;
    ib = jb;
}

template <typename T>
__device__ __forceinline__ T median25(const T* __restrict__ p, int h, int w, int y, int x, int* src)
{
    T v[32];
    int id[32];
#pragma unroll
    for (int dy = 0; dy < 5; ++dy) {
        int yy = y + dy - 2;
        yy = yy < 0 ? -yy : (yy > h - 1 ? 2 * (h - 1) - yy : yy);
#pragma unroll
        for (int dx = 0; dx < 5; ++dx) {
            int xx = x + dx - 2;
            xx = xx < 0 ? -xx : (xx > w - 1 ? 2 * (w - 1) - xx : xx);
            id[dy * 5 + dx] = yy * w + xx;
            v[dy * 5 + dx] = p[id[dy * 5 + dx]];
        }
    }
#pragma unroll
    for (int i = 25; i < 32; ++i) {
        v[i] = (T)INFINITY;
        id[i] = -1;
    }
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const int l = i ^ j;
                if (l > i) cswap(v[i], v[l], id[i], id[l], (i & k) == 0);
            }
    if (src) *src = id[12];
    return v[12];
}

// uv_out = uv_in + (median ? median5(d) : d) on the two planes of each frame.
template <typename T>
__global__ void kd_median_add(const T* __restrict__ d, const T* __restrict__ uv_in, T* __restrict__ uv_out, int h,
                              int w, int median)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long pl = blockIdx.z, hw = (long long)h * w, pix = (long long)y * w + x;
    const T* p = d + pl * hw;
    const T m = median ? median25(p, h, w, y, x, (int*)nullptr) : p[pix];
    uv_out[pl * hw + pix] = uv_in[pl * hw + pix] + m;
}

template <typename T>
__global__ void kd_argmedian(const T* __restrict__ d, int h, int w, int32_t* __restrict__ am)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long pl = blockIdx.z, hw = (long long)h * w;
    int s = 0;
    median25(d + pl * hw, h, w, y, x, &s);
    am[pl * hw + (long long)y * w + x] = s;
}

// g_d(q) = sum of g(p) over the windows p whose median came from q; with
// mirror borders those windows lie within two pixels of q on each axis.
template <typename T>
__global__ void kd_median_adj(const int32_t* __restrict__ am, const T* __restrict__ g, int h, int w,
                              T* __restrict__ gd)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) return;
    const int y = blockIdx.y;
    const long long pl = blockIdx.z, hw = (long long)h * w;
    const int q = y * w + x;
    T acc = 0;
    for (int py = (y > 2 ? y - 2 : 0); py <= (y + 2 < h - 1 ? y + 2 : h - 1); ++py)
        for (int px = (x > 2 ? x - 2 : 0); px <= (x + 2 < w - 1 ? x + 2 : w - 1); ++px) {
            const long long p = pl * hw + (long long)py * w + px;
            if (am[p] == q) acc += g[p];
        }
    gd[pl * hw + q] = acc;
}

dim3 grid_rows(int w, int h, long long planes, int bx = 128)
{
    return dim3((unsigned)((w + bx - 1) / bx), (unsigned)h, (unsigned)planes);
}

}  // namespace

// ------------------------------------------------------------------ launchers
template <typename T>
cudaError_t resize(const T* src, long long planes, int ih, int iw, int oh, int ow, const int32_t* ix, const float* wx,
                   int Px, const int32_t* iy, const float* wy, int Py, T* tmp, T* dst, cudaStream_t st)
{
    kd_resize_h<T><<<grid_rows(ow, ih, planes), 128, 0, st>>>(src, ih, iw, ow, ix, wx, Px, tmp);
    kd_resize_v<T><<<grid_rows(ow, oh, planes), 128, 0, st>>>(tmp, ih, ow, oh, iy, wy, Py, dst);
    return cudaGetLastError();
}

template <typename T>
cudaError_t resize_t(const T* gdst, long long planes, int oh, int ow, int ih, int iw, const Csr& cx, const Csr& cy,
                     T* tmp, T* gsrc, int accumulate, cudaStream_t st)
{
    kd_resize_vt<T><<<grid_rows(ow, ih, planes), 128, 0, st>>>(gdst, oh, ow, ih, cy.ptr, cy.idx, cy.w, tmp);
    kd_resize_ht<T><<<grid_rows(iw, ih, planes), 128, 0, st>>>(tmp, ih, ow, iw, cx.ptr, cx.idx, cx.w, gsrc,
                                                               accumulate);
    return cudaGetLastError();
}

template <typename T>
cudaError_t warp(const T* f2, const T* f1, const T* uv, int F, int K, int h, int w, double hcol, double hrow, T* out,
                 cudaStream_t st)
{
    kd_warp<T><<<grid_rows(w, h, F), 128, 0, st>>>(f2, f1, uv, K, h, w, (T)hcol, (T)hrow, out);
    return cudaGetLastError();
}

template <typename T>
cudaError_t warp_adj(const T* f2, const T* uv, const T* gout, int F, int K, int h, int w, double hcol, double hrow,
                     T* gf2, T* gf1, T* guv, cudaStream_t st)
{
    kd_warp_adj<T><<<grid_rows(w, h, F), 128, 0, st>>>(f2, uv, gout, K, h, w, (T)hcol, (T)hrow, gf2, gf1, guv);
    return cudaGetLastError();
}

template <typename T>
cudaError_t tensor(const T* f1, const T* f2, int F, int K, int h, int w, double hy, double hx, T* J, cudaStream_t st)
{
    kd_tensor<T><<<grid_rows(w, h, (long long)F * K), 128, 0, st>>>(f1, f2, K, h, w, (T)hy, (T)hx, J);
    return cudaGetLastError();
}

template <typename T>
cudaError_t tensor_adj(const T* f1, const T* f2, const T* gJ, int F, int K, int h, int w, double hy, double hx, T* G,
                       T* gf1, T* gf2, int accumulate_f1, cudaStream_t st)
{
    kd_tensor_adj_local<T><<<grid_rows(w, h, (long long)F * K), 128, 0, st>>>(f1, f2, gJ, K, h, w, (T)hy, (T)hx, G);
    kd_tensor_adj_gather<T><<<grid_rows(w, h, (long long)F * K), 128, 0, st>>>(G, K, h, w, (T)hy, (T)hx, gf1, gf2,
                                                                               accumulate_f1);
    return cudaGetLastError();
}

template <typename T>
cudaError_t tick(const T* J, const T* W, const T* stt, const T* uv, int F, int K, int h, int w, const double* a_data,
                 double eps, double ax, double ay, T* coef, T* ck, cudaStream_t st)
{
    AData ad;
    for (int k = 0; k < kMaxK; ++k) ad.a[k] = k < K ? a_data[k] : 0.0;
    kd_tick<T><<<grid_rows(w, h, F), 128, 0, st>>>(J, W, stt, uv, K, h, w, ad, (T)eps, (T)ax, (T)ay, coef, ck);
    return cudaGetLastError();
}

template <typename T>
cudaError_t rb_sweep(int color, const T* coef, const T* rhs, T* state, T* store, int F, int h, int w, double ax,
                     double ay, double omega, double eps, int gs, cudaStream_t st)
{
    kd_rb_sweep<T><<<grid_rows((w + 1) / 2, h, F), 128, 0, st>>>(color, coef, rhs, state, store, h, w, (T)ax, (T)ay,
                                                                 (T)omega, (T)eps, gs);
    return cudaGetLastError();
}

template <typename T>
cudaError_t implicit_assemble(const T* lam, const T* x, int F, int h, int w, T* gcoef, double sx, double sy,
                              double* galpha, cudaStream_t st)
{
    kd_implicit_assemble<T><<<grid_rows(w, h, F), 128, 0, st>>>(lam, x, h, w, gcoef, sx, sy, galpha);
    return cudaGetLastError();
}

template <typename T>
cudaError_t rb_adj_step(int color, const T* coef, const T* pre_full, const T* pre_c0, const T* pre_c1, T* lam,
                        const T* aprev, T* anext, int F, int h, int w, double ax, double ay, double omega, double eps,
                        int gs, T* gcoef, double sx, double sy, double* galpha, cudaStream_t st)
{
    StateSrc<T> pre{pre_full, pre_c0, pre_c1};
    kd_rb_adj_step<T><<<grid_rows((w + 1) / 2, h, F), 128, 0, st>>>(color, coef, pre, lam, aprev, anext, h, w, (T)ax,
                                                                    (T)ay, (T)omega, (T)eps, gs, gcoef, sx, sy,
                                                                    galpha);
    return cudaGetLastError();
}

// Shared memory of kd_rb_adj_window for square tiles of edge t and windows of
// nh half-sweeps: 9 planes over the tile grown by nh, 4 state planes (2 per
// colour buffer pair, half a plane each) over the tile grown by nh + 1, and
// the two colours' ring tables (one int2 per pixel of the tile grown by nh).
size_t adj_window_smem(int t, int nh, int elem_bytes)
{
    const size_t r = (size_t)(t + 2 * nh) * (t + 2 * nh), r1 = (size_t)(t + 2 * nh + 2) * (t + 2 * nh + 2);
    return (9 * r + 4 * r1) * elem_bytes + r * sizeof(int2);  // planes, state buffers, ring tables
}

// The ring tables of kd_rb_adj_window for square tiles of edge t and windows
// of nh half-sweeps, on the host: per colour c the offsets (dx, dy) from the
// tile origin of the pixels of that colour within nh of the tile ((dx + dy)
// & 1 == c: tile origins are even), the tile's own first (entry k: the pixel
// of colour c of thread k's pair, row k / (t / 2), columns 2 (k % (t / 2)) and
// one right), then ring by ring; cnt[c][d] = entries within distance d.
// Entry: x = (dy << 16) | (dx & 0xffff); y = li | sb << 13 | p << 26 with li
// the pixel in the planes over the tile grown by nh, sb its pair in the state
// buffers over the tile grown by nh + 1 and p its column parity in the pair.
bool build_adj_table(int t, int nh, std::vector<int2>& e0, std::vector<int2>& e1, int cnt[2][kAdjMaxNh + 1])
{
    if (nh < 1 || nh > kAdjMaxNh || (t & 1)) return false;
    const int Rw = t + 2 * nh, Rp1 = (Rw + 2) / 2;
    if (Rw * Rw >= (1 << 13) || (Rw + 2) * Rp1 >= (1 << 13)) return false;
    auto enc = [&](int dx, int dy) {
        const int li = (dy + nh) * Rw + (dx + nh);
        const int sb = (dy + nh + 1) * Rp1 + ((dx + nh + 1) >> 1);
        const int p = (dx + nh + 1) & 1;
        return make_int2((int)(((unsigned)dy << 16) | ((unsigned)dx & 0xffffu)), li | (sb << 13) | (p << 26));
    };
    for (int c = 0; c < 2; ++c) {
        std::vector<int2>& e = c == 0 ? e0 : e1;
        e.clear();
        for (int k = 0; k < t * t / 2; ++k) {
            const int oy = k / (t / 2), ox = 2 * (k % (t / 2));
            const int dx = ox + ((c - ox - oy) & 1);
            e.push_back(enc(dx, oy));
        }
        cnt[c][0] = (int)e.size();
        for (int d = 1; d <= nh; ++d) {
            for (int dy = -d; dy < t + d; ++dy)
                for (int dx = -d; dx < t + d; ++dx) {
                    const int dist = std::max(std::max(-dx, dx - (t - 1)), std::max(-dy, dy - (t - 1)));
                    if (dist == d && ((dx + dy) & 1) == c) e.push_back(enc(dx, dy));
                }
            cnt[c][d] = (int)e.size();
        }
    }
    return true;
}

// Tile edge of kd_rb_adj_window for windows of nh half-sweeps: 32 or 16, the
// largest whose shared memory fits; 0 when none does (the window then runs one
// launch per half-sweep).
int rb_adj_window_tile(int nh, int elem_bytes)
{
    for (int t : {32, 16})
        if (adj_window_smem(t, nh, elem_bytes) <= kAdjWindowSmem) return t;
    return 0;
}

template <typename T>
cudaError_t rb_adj_window(const T* coef, const T* s0, const T* hist, long long slot, const T* lam_in, T* lam_out,
                          int F, int h, int w, int nh, int tile, const AdjTable& tab, double ax, double ay,
                          double omega, double eps, int gs, T* gcoef, double sx, double sy, double* galpha,
                          cudaStream_t st)
{
    const size_t bytes = adj_window_smem(tile, nh, (int)sizeof(T));
    if ((tile != 16 && tile != 32) || nh < 1 || bytes > kAdjWindowSmem) return cudaErrorInvalidValue;
    const cudaError_t e = ensure_max_dyn_smem((const void*)kd_rb_adj_window<T>, (int)kAdjWindowSmem);
    if (e != cudaSuccess) return e;
    const dim3 grid((w + tile - 1) / tile, (h + tile - 1) / tile, F);
    kd_rb_adj_window<T><<<grid, tile * tile / 2, bytes, st>>>(coef, s0, hist, slot, lam_in, lam_out, h, w, nh, tile,
                                                             tile, tab, (T)ax, (T)ay, (T)omega, (T)eps, gs, gcoef, sx,
                                                             sy, galpha);
    return cudaGetLastError();
}

cudaError_t reduce_slots(double* part, int F, long long n_slots, double* galpha, cudaStream_t st)
{
    kd_reduce_slots<<<F, 256, 0, st>>>(part, n_slots, galpha);
    return cudaGetLastError();
}

template <typename T>
cudaError_t rb_adj_gather(int color, T* lam, const T* aprev, int F, int h, int w, double ax, double ay,
                          cudaStream_t st)
{
    kd_rb_adj_gather<T><<<grid_rows((w + 1) / 2, h, F), 128, 0, st>>>(color, lam, aprev, h, w, (T)ax, (T)ay);
    return cudaGetLastError();
}

template <typename T>
cudaError_t tick_adj(const T* J, const T* W, const T* stt, const T* uv, const T* gcoef, int F, int K, int h, int w,
                     const double* a_data, double eps, double ax, double ay, int lagged, T* gJ, T* lam, T* guv,
                     double sx, double sy, double* galpha, cudaStream_t st)
{
    AData ad;
    for (int k = 0; k < kMaxK; ++k) ad.a[k] = k < K ? a_data[k] : 0.0;
    const dim3 grid = grid_rows(w, h, F);
    if (K == 1)
        kd_tick_adj<T, 1><<<grid, 128, 0, st>>>(J, W, stt, uv, gcoef, K, h, w, ad, (T)eps, (T)ax, (T)ay, lagged, gJ,
                                                lam, guv, sx, sy, galpha);
    else if (K == 2)
        kd_tick_adj<T, 2><<<grid, 128, 0, st>>>(J, W, stt, uv, gcoef, K, h, w, ad, (T)eps, (T)ax, (T)ay, lagged, gJ,
                                                lam, guv, sx, sy, galpha);
    else
        kd_tick_adj<T, 0><<<grid, 128, 0, st>>>(J, W, stt, uv, gcoef, K, h, w, ad, (T)eps, (T)ax, (T)ay, lagged, gJ,
                                                lam, guv, sx, sy, galpha);
    return cudaGetLastError();
}

template <typename T>
cudaError_t median_add(const T* d, const T* uv_in, T* uv_out, int F, int h, int w, int median, cudaStream_t st)
{
    kd_median_add<T><<<grid_rows(w, h, (long long)F * 2), 128, 0, st>>>(d, uv_in, uv_out, h, w, median);
    return cudaGetLastError();
}

template <typename T>
cudaError_t median_adj(const T* d, const T* g, int32_t* am, int F, int h, int w, T* gd, cudaStream_t st)
{
    kd_argmedian<T><<<grid_rows(w, h, (long long)F * 2), 128, 0, st>>>(d, h, w, am);
    kd_median_adj<T><<<grid_rows(w, h, (long long)F * 2), 128, 0, st>>>(am, g, h, w, gd);
    return cudaGetLastError();
}

#define FRG_DIFF_INSTANTIATE(T)                                                                                 \
    template cudaError_t resize<T>(const T*, long long, int, int, int, int, const int32_t*, const float*, int,   \
                                   const int32_t*, const float*, int, T*, T*, cudaStream_t);                    \
    template cudaError_t resize_t<T>(const T*, long long, int, int, int, int, const Csr&, const Csr&, T*, T*,     \
                                     int, cudaStream_t);                                                        \
    template cudaError_t warp<T>(const T*, const T*, const T*, int, int, int, int, double, double, T*,           \
                                 cudaStream_t);                                                                 \
    template cudaError_t warp_adj<T>(const T*, const T*, const T*, int, int, int, int, double, double, T*, T*,   \
                                     T*, cudaStream_t);                                                         \
    template cudaError_t tensor<T>(const T*, const T*, int, int, int, int, double, double, T*, cudaStream_t);   \
    template cudaError_t tensor_adj<T>(const T*, const T*, const T*, int, int, int, int, double, double, T*, T*, \
                                       T*, int, cudaStream_t);                                                  \
    template cudaError_t tick<T>(const T*, const T*, const T*, const T*, int, int, int, int, const double*,      \
                                 double, double, double, T*, T*, cudaStream_t);                                 \
    template cudaError_t rb_sweep<T>(int, const T*, const T*, T*, T*, int, int, int, double, double, double,     \
                                     double, int, cudaStream_t);                                                \
    template cudaError_t implicit_assemble<T>(const T*, const T*, int, int, int, T*, double, double, double*,    \
                                              cudaStream_t);                                                    \
    template cudaError_t rb_adj_step<T>(int, const T*, const T*, const T*, const T*, T*, const T*, T*, int, int, \
                                        int, double, double, double, double, int, T*, double, double, double*,  \
                                        cudaStream_t);                                                          \
    template cudaError_t rb_adj_gather<T>(int, T*, const T*, int, int, int, double, double, cudaStream_t);      \
    template cudaError_t rb_adj_window<T>(const T*, const T*, const T*, long long, const T*, T*, int, int, int, int,  \
                                          int, const AdjTable&, double, double, double, double, int, T*, double,     \
                                          double, double*, cudaStream_t);                                             \
    template cudaError_t tick_adj<T>(const T*, const T*, const T*, const T*, const T*, int, int, int, int,       \
                                     const double*, double, double, double, int, T*, T*, T*, double, double,    \
                                     double*, cudaStream_t);                                                    \
    template cudaError_t median_add<T>(const T*, const T*, T*, int, int, int, int, cudaStream_t);               \
    template cudaError_t median_adj<T>(const T*, const T*, int32_t*, int, int, int, T*, cudaStream_t);

FRG_DIFF_INSTANTIATE(float)
FRG_DIFF_INSTANTIATE(double)

}  // namespace diff
}  // namespace frg
