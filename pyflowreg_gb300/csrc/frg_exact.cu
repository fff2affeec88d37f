// FP64 reference-order kernels (parity mode).
//
// These follow the numba typing of pyflowreg's arithmetic operation by
// operation -- float32 images and resize products, float64 accumulators,
// tensors and solver -- with explicit round-to-nearest intrinsics so that no
// multiply-add is contracted.  They share the schedule, the tap tables and the
// exact lexicographic SOR order with the FP32 path; their purpose is to show
// that the GB300 pipeline reproduces the reference's result to within the
// reference's own rounding when it computes in the reference's precision.
// Layout: row-major planes, the level arrays with their one-pixel ring
// (m = h + 2 rows, n = w + 2 columns), like the reference's numpy arrays.
#include "frg_internal.h"
#include "frg_select.cuh"

#include <math.h>

namespace frg {

__device__ __forceinline__ int xclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// float -> double on the integer pipe: the conversion instruction runs on the
// float64 pipe (GB300: 1/64 of the float32 rate), while a normal float's bits
// map to the double's by a re-biased exponent and a shifted fraction.  Exact;
// zeros likewise; subnormals, infinities and NaN take the conversion.
__device__ __forceinline__ double f2d(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) {
        if ((b << 1) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
        return (double)f;
    }
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b >> 3) & 0xfffffu);
    return __hiloint2double((int)hi, (int)(b << 29));
}

// ---------------------------------------------------------------------------
// Resize with numba typing (util/resize_util.py:116-141): float32 input and
// products, float64 accumulator, float32 result (stored as float or double).
// ---------------------------------------------------------------------------
template <typename Tin>
__global__ void kx_resize_h(const Tin* __restrict__ src, long long fs, long long ps, long long rs, long long cs,
                            int n_planes, int ih, float* __restrict__ dst, int ow, const int32_t* __restrict__ ix,
                            const float* __restrict__ wx, int P)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int fp = blockIdx.z;
    if (x >= ow) return;
    const int f = fp / n_planes, pl = fp - f * n_planes;
    const Tin* row = src + f * fs + pl * ps + (long long)y * rs;
    double s = 0.0;
    for (int p = 0; p < P; ++p) {
        const float a = (float)row[(long long)ix[(long long)x * P + p] * cs];
        s = dadd(s, f2d(__fmul_rn(a, wx[(long long)x * P + p])));
    }
    dst[((long long)fp * ih + y) * ow + x] = (float)s;
}

// ring: 0 none, 1 edge-replicated ring (add_boundary), 2 zero ring
// (cv2.copyMakeBorder BORDER_CONSTANT 0, core/optical_flow.py:565-568).
template <typename Tout>
__global__ void kx_resize_v(const float* __restrict__ src, int n_planes, int ih, int ow, Tout* __restrict__ dst,
                            long long fs, long long ps, long long rs, int oh, int ring,
                            const int32_t* __restrict__ iy, const float* __restrict__ wy, int P)
{
    const int pad = ring ? 1 : 0;
    const int xo = blockIdx.x * blockDim.x + threadIdx.x;
    const int yo = blockIdx.y;
    const int fp = blockIdx.z;
    if (xo >= ow + 2 * pad) return;
    const int f = fp / n_planes, pl = fp - f * n_planes;
    Tout* out = dst + f * fs + pl * ps + (long long)yo * rs + xo;
    const bool inside = xo >= pad && xo < ow + pad && yo >= pad && yo < oh + pad;
    if (!inside && ring == 2) {
        *out = (Tout)0;
        return;
    }
    const int x = xclamp(xo - pad, 0, ow - 1);
    const int y = xclamp(yo - pad, 0, oh - 1);
    const float* col = src + (long long)fp * ih * ow + x;
    double s = 0.0;
    for (int p = 0; p < P; ++p)
        s = dadd(s, f2d(__fmul_rn(col[(long long)iy[(long long)y * P + p] * ow], wy[(long long)y * P + p])));
    *out = (Tout)(float)s;
}

cudaError_t launch_x_resize_h_f(const float* src, long long fs, long long ps, long long rs, long long cs,
                                int n_frames, int n_planes, int ih, float* dst, int ow, const int32_t* ix,
                                const float* wx, int P, cudaStream_t st)
{
    dim3 blk(128), grd((ow + 127) / 128, ih, n_frames * n_planes);
    kx_resize_h<float><<<grd, blk, 0, st>>>(src, fs, ps, rs, cs, n_planes, ih, dst, ow, ix, wx, P);
    return cudaGetLastError();
}

cudaError_t launch_x_resize_h_d(const double* src, long long fs, long long ps, long long rs, long long cs,
                                int n_frames, int n_planes, int ih, float* dst, int ow, const int32_t* ix,
                                const float* wx, int P, cudaStream_t st)
{
    dim3 blk(128), grd((ow + 127) / 128, ih, n_frames * n_planes);
    kx_resize_h<double><<<grd, blk, 0, st>>>(src, fs, ps, rs, cs, n_planes, ih, dst, ow, ix, wx, P);
    return cudaGetLastError();
}

cudaError_t launch_x_resize_v_f(const float* src, int n_frames, int n_planes, int ih, int ow, float* dst,
                                long long fs, long long ps, long long rs, int oh, int ring, const int32_t* iy,
                                const float* wy, int P, cudaStream_t st)
{
    const int pad = ring ? 1 : 0;
    dim3 blk(128), grd((ow + 2 * pad + 127) / 128, oh + 2 * pad, n_frames * n_planes);
    kx_resize_v<float><<<grd, blk, 0, st>>>(src, n_planes, ih, ow, dst, fs, ps, rs, oh, ring, iy, wy, P);
    return cudaGetLastError();
}

cudaError_t launch_x_resize_v_d(const float* src, int n_frames, int n_planes, int ih, int ow, double* dst,
                                long long fs, long long ps, long long rs, int oh, int ring, const int32_t* iy,
                                const float* wy, int P, cudaStream_t st)
{
    const int pad = ring ? 1 : 0;
    dim3 blk(128), grd((ow + 2 * pad + 127) / 128, oh + 2 * pad, n_frames * n_planes);
    kx_resize_v<double><<<grd, blk, 0, st>>>(src, n_planes, ih, ow, dst, fs, ps, rs, oh, ring, iy, wy, P);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Warp (core/warping.py:160-234) with float64 flow: map = float32(x + u/h_col),
// float64 accumulation of float32 weights, float32 result.
// u, v: padded (m, n) planes, frame stride uv_fs.  f2: (T, K, h, w) float,
// f1: (K, h, w) float shared, out (T, K, h, w) float.
// ---------------------------------------------------------------------------
__constant__ float cx_cubic[32 * 4];

cudaError_t upload_cubic_table_x(const float* tab128)
{
    return cudaMemcpyToSymbol(cx_cubic, tab128, sizeof(float) * 128);
}

// The flow over the spacing: a product with the reciprocal where the spacing is a
// power of two (the finest level's 1), which rounds like the quotient.
struct WarpScale {
    double h_col, h_row, i_col, i_row;
    int pow2_col, pow2_row;
};

__global__ void kx_warp(const float* __restrict__ f2, const float* __restrict__ f1, const double* __restrict__ u,
                        const double* __restrict__ v, long long uv_fs, int K, int h, int w, WarpScale S,
                        float* __restrict__ out)
{
    // the table is read per lane at the lane's own sub-pixel position: copied into shared
    // memory first (constant memory serialises a warp's distinct addresses)
    __shared__ float s_tab[32 * 4];
    for (int i = threadIdx.x; i < 32 * 4; i += blockDim.x) s_tab[i] = cx_cubic[i];
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int f = blockIdx.z;
    if (x >= w) return;
    const long long n = w + 2;
    const long long hw = (long long)h * w;
    const long long o = (long long)(y + 1) * n + (x + 1);
    const double uu = u[f * uv_fs + o], vv = v[f * uv_fs + o];
    const float mx = (float)dadd((double)x, S.pow2_col ? dmul(uu, S.i_col) : ddiv(uu, S.h_col));
    const float my = (float)dadd((double)y, S.pow2_row ? dmul(vv, S.i_row) : ddiv(vv, S.h_row));
    const bool oob = (mx < 0.0f) || (mx >= (float)w) || (my < 0.0f) || (my >= (float)h);
    if (oob) {
        for (int k = 0; k < K; ++k)
            out[((long long)f * K + k) * hw + (long long)y * w + x] = f1[(long long)k * hw + (long long)y * w + x];
        return;
    }
    const float cx = fminf(fmaxf(mx, 0.0f), (float)(w - 1));
    const float cy = fminf(fmaxf(my, 0.0f), (float)(h - 1));
    const int X = __float2int_rn(cx * 32.0f), Y = __float2int_rn(cy * 32.0f);
    const int ix = X >> 5, fx = X & 31, iy = Y >> 5, fy = Y & 31;
    // the 16 weights (float products, exact in double) and the tap offsets, once for all channels
    double w2[4][4];
    long long ro[4];
    int co[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float wyi = s_tab[fy * 4 + i];
#pragma unroll
        for (int j = 0; j < 4; ++j) w2[i][j] = f2d(__fmul_rn(wyi, s_tab[fx * 4 + j]));
        ro[i] = (long long)xclamp(iy - 1 + i, 0, h - 1) * w;
        co[i] = xclamp(ix - 1 + i, 0, w - 1);
    }
    for (int k = 0; k < K; ++k) {
        const float* src = f2 + ((long long)f * K + k) * hw;
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
                // the product of two floats is exact in double, so the fused form rounds as
                // dadd(acc, dmul(...)) does
                acc = __fma_rn(f2d(src[ro[i] + co[j]]), w2[i][j], acc);
        out[((long long)f * K + k) * hw + (long long)y * w + x] = (float)acc;
    }
}

cudaError_t launch_x_warp(const float* f2, const float* f1, const double* u, const double* v, long long uv_fs,
                          int n_frames, int K, int h, int w, double h_col, double h_row, float* out, cudaStream_t st)
{
    WarpScale S;
    S.h_col = h_col;
    S.h_row = h_row;
    int ex = 0;
    S.pow2_col = frexp(h_col, &ex) == 0.5 ? 1 : 0;
    S.pow2_row = frexp(h_row, &ex) == 0.5 ? 1 : 0;
    S.i_col = 1.0 / h_col;
    S.i_row = 1.0 / h_row;
    dim3 blk(128), grd((w + 127) / 128, h, n_frames);
    kx_warp<<<grd, blk, 0, st>>>(f2, f1, u, v, uv_fs, K, h, w, S, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Motion tensor (core/optical_flow.py:73-228), the oracle's arithmetic:
// float64, except that the derivatives of the warped image are float32
// (numpy keeps a float32 array float32 under a Python-float spacing) when
// f2_f32 is set (every level below the top).
// f1: (K, h, w) float shared; f2: (T, K, h, w) float; J: (T, 6, K, m*n) double
// with a zero ring.
// ---------------------------------------------------------------------------
// J11..J23 of channel k at padded position (yo, xo) (interior: 1..h, 1..w):
// the oracle's arithmetic, operation by operation.
__device__ __forceinline__ void tensor_px64(const float* __restrict__ f1, const float* __restrict__ f2, int f, int K,
                                            int k, int h, int w, int yo, int xo, double hy, double hx, int f2_f32,
                                            int gray, double* jo)
{
    const long long hw = (long long)h * w;
    const double h2x = dmul(2.0, hx), h2y = dmul(2.0, hy), hxx = dmul(hx, hx), hyy = dmul(hy, hy);
    const float h2x_f = (float)h2x, h2y_f = (float)h2y;
    const float hxx_f = (float)hxx, hyy_f = (float)hyy;
    const float* a = f1 + (long long)k * hw;
    const float* b = f2 + ((long long)f * K + k) * hw;
    // padded (yy, xx) -> unpadded clamp
    auto A = [&](int yy, int xx) { return (double)a[(long long)xclamp(yy - 1, 0, h - 1) * w + xclamp(xx - 1, 0, w - 1)]; };
    auto Bf = [&](int yy, int xx) { return b[(long long)xclamp(yy - 1, 0, h - 1) * w + xclamp(xx - 1, 0, w - 1)]; };
    // numpy.gradient of the padded arrays at an interior padded position
    auto gx1 = [&](int yy, int xx) { return ddiv(dsub(A(yy, xx + 1), A(yy, xx - 1)), h2x); };
    auto gy1 = [&](int yy, int xx) { return ddiv(dsub(A(yy + 1, xx), A(yy - 1, xx)), h2y); };
    auto gx2 = [&](int yy, int xx) {
        if (f2_f32) return (double)__fdiv_rn(__fsub_rn(Bf(yy, xx + 1), Bf(yy, xx - 1)), h2x_f);
        return ddiv(dsub((double)Bf(yy, xx + 1), (double)Bf(yy, xx - 1)), h2x);
    };
    auto gy2 = [&](int yy, int xx) {
        if (f2_f32) return (double)__fdiv_rn(__fsub_rn(Bf(yy + 1, xx), Bf(yy - 1, xx)), h2y_f);
        return ddiv(dsub((double)Bf(yy + 1, xx), (double)Bf(yy - 1, xx)), h2y);
    };
    // fx, fy, ft re-padded from the interior: clamp the padded index to [1, h] x [1, w]
    auto FX = [&](int yy, int xx) {
        yy = xclamp(yy, 1, h);
        xx = xclamp(xx, 1, w);
        return dmul(0.5, dadd(gx1(yy, xx), gx2(yy, xx)));
    };
    auto FT = [&](int yy, int xx) {
        yy = xclamp(yy, 1, h);
        xx = xclamp(xx, 1, w);
        return dsub((double)Bf(yy, xx), A(yy, xx));
    };
    double j11, j22, j33, j12, j13, j23;
    if (gray == 2) {
        // census (core/optical_flow.py:231-345): per neighbour offset the smoothed
        // Heaviside of the directional difference, s = 0.5 (1 + r / sqrt(r^2 + eps^2)),
        // edge-padded, differentiated centrally; float32 arithmetic on f2 when
        // f2_f32 (Python-float constants cast to float32), float64 otherwise
        const double eps = 0.1 / 255.0, eps2 = dmul(eps, eps);
        const float eps2f = (float)eps2;
        j11 = j22 = j33 = j12 = j13 = j23 = 0.0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                if (dy == 0 && dx == 0) continue;
                const double ty = dmul(hy, (double)dy), tx = dmul(hx, (double)dx);
                const double dist = __dsqrt_rn(dadd(dmul(ty, ty), dmul(tx, tx)));
                const float dist_f = (float)dist;
                // s at padded (yy, xx), the edge pad of the core (clamped into [1, h] x [1, w])
                auto s1 = [&](int yy, int xx) {
                    yy = xclamp(yy, 1, h);
                    xx = xclamp(xx, 1, w);
                    const double r = ddiv(dsub(A(yy + dy, xx + dx), A(yy, xx)), dist);
                    return dmul(0.5, dadd(1.0, ddiv(r, __dsqrt_rn(dadd(dmul(r, r), eps2)))));
                };
                auto s2 = [&](int yy, int xx) {
                    yy = xclamp(yy, 1, h);
                    xx = xclamp(xx, 1, w);
                    if (f2_f32) {
                        const float r = __fdiv_rn(__fsub_rn(Bf(yy + dy, xx + dx), Bf(yy, xx)), dist_f);
                        const float q = __fsqrt_rn(__fadd_rn(__fmul_rn(r, r), eps2f));
                        return (double)__fmul_rn(0.5f, __fadd_rn(1.0f, __fdiv_rn(r, q)));
                    }
                    const double r = ddiv(dsub((double)Bf(yy + dy, xx + dx), (double)Bf(yy, xx)), dist);
                    return dmul(0.5, dadd(1.0, ddiv(r, __dsqrt_rn(dadd(dmul(r, r), eps2)))));
                };
                const double sx1 = ddiv(dsub(s1(yo, xo + 1), s1(yo, xo - 1)), h2x);
                const double sy1 = ddiv(dsub(s1(yo + 1, xo), s1(yo - 1, xo)), h2y);
                double sx2, sy2;
                if (f2_f32) {
                    sx2 = (double)__fdiv_rn(__fsub_rn((float)s2(yo, xo + 1), (float)s2(yo, xo - 1)), h2x_f);
                    sy2 = (double)__fdiv_rn(__fsub_rn((float)s2(yo + 1, xo), (float)s2(yo - 1, xo)), h2y_f);
                } else {
                    sx2 = ddiv(dsub(s2(yo, xo + 1), s2(yo, xo - 1)), h2x);
                    sy2 = ddiv(dsub(s2(yo + 1, xo), s2(yo - 1, xo)), h2y);
                }
                const double sx = dmul(0.5, dadd(sx1, sx2)), sy = dmul(0.5, dadd(sy1, sy2));
                const double st = dsub(s2(yo, xo), s1(yo, xo));
                j11 = dadd(j11, dmul(sx, sx));
                j22 = dadd(j22, dmul(sy, sy));
                j33 = dadd(j33, dmul(st, st));
                j12 = dadd(j12, dmul(sx, sy));
                j13 = dadd(j13, dmul(sx, st));
                j23 = dadd(j23, dmul(sy, st));
            }
        j11 = dmul(j11, 0.25); j22 = dmul(j22, 0.25); j33 = dmul(j33, 0.25);
        j12 = dmul(j12, 0.25); j13 = dmul(j13, 0.25); j23 = dmul(j23, 0.25);
    } else if (gray) {
        const double fxv = FX(yo, xo);
        const double fyv = dmul(0.5, dadd(gy1(yo, xo), gy2(yo, xo)));
        const double ftv = FT(yo, xo);
        j11 = dmul(fxv, fxv); j22 = dmul(fyv, fyv); j33 = dmul(ftv, ftv);
        j12 = dmul(fxv, fyv); j13 = dmul(fxv, ftv); j23 = dmul(fyv, ftv);
    } else {
        const double fxy = ddiv(dsub(FX(yo + 1, xo), FX(yo - 1, xo)), h2y);
        const double fxt = ddiv(dsub(FT(yo, xo + 1), FT(yo, xo - 1)), h2x);
        const double fyt = ddiv(dsub(FT(yo + 1, xo), FT(yo - 1, xo)), h2y);
        const double fxx1 = ddiv(dadd(dsub(A(yo, xo - 1), dmul(2.0, A(yo, xo))), A(yo, xo + 1)), hxx);
        const double fyy1 = ddiv(dadd(dsub(A(yo - 1, xo), dmul(2.0, A(yo, xo))), A(yo + 1, xo)), hyy);
        double fxx2, fyy2;
        if (f2_f32) {
            fxx2 = (double)__fdiv_rn(__fadd_rn(__fsub_rn(Bf(yo, xo - 1), __fmul_rn(2.0f, Bf(yo, xo))), Bf(yo, xo + 1)), hxx_f);
            fyy2 = (double)__fdiv_rn(__fadd_rn(__fsub_rn(Bf(yo - 1, xo), __fmul_rn(2.0f, Bf(yo, xo))), Bf(yo + 1, xo)), hyy_f);
        } else {
            fxx2 = ddiv(dadd(dsub((double)Bf(yo, xo - 1), dmul(2.0, (double)Bf(yo, xo))), (double)Bf(yo, xo + 1)), hxx);
            fyy2 = ddiv(dadd(dsub((double)Bf(yo - 1, xo), dmul(2.0, (double)Bf(yo, xo))), (double)Bf(yo + 1, xo)), hyy);
        }
        const double fxx = dmul(0.5, dadd(fxx1, fxx2));
        const double fyy = dmul(0.5, dadd(fyy1, fyy2));
        const double sx = __dsqrt_rn(dadd(dmul(fxx, fxx), dmul(fxy, fxy)));
        const double sy = __dsqrt_rn(dadd(dmul(fxy, fxy), dmul(fyy, fyy)));
        const double reg_x = ddiv(1.0, dadd(dmul(sx, sx), 1e-6));
        const double reg_y = ddiv(1.0, dadd(dmul(sy, sy), 1e-6));
        j11 = dadd(dmul(reg_x, dmul(fxx, fxx)), dmul(reg_y, dmul(fxy, fxy)));
        j22 = dadd(dmul(reg_x, dmul(fxy, fxy)), dmul(reg_y, dmul(fyy, fyy)));
        j33 = dadd(dmul(reg_x, dmul(fxt, fxt)), dmul(reg_y, dmul(fyt, fyt)));
        j12 = dadd(dmul(dmul(reg_x, fxx), fxy), dmul(dmul(reg_y, fxy), fyy));
        j13 = dadd(dmul(dmul(reg_x, fxx), fxt), dmul(dmul(reg_y, fxy), fyt));
        j23 = dadd(dmul(dmul(reg_x, fxy), fxt), dmul(dmul(reg_y, fyy), fyt));
    }
    jo[0] = j11;
    jo[1] = j22;
    jo[2] = j33;
    jo[3] = j12;
    jo[4] = j13;
    jo[5] = j23;
}

__global__ void kx_tensor(const float* __restrict__ f1, const float* __restrict__ f2, int K, int h, int w,
                          double hy, double hx, int f2_f32, int gray, double* __restrict__ J)
{
    const int xo = blockIdx.x * blockDim.x + threadIdx.x;  // padded column
    const int yo = blockIdx.y;                             // padded row
    const int f = blockIdx.z;
    const int n = w + 2, m = h + 2;
    if (xo >= n) return;
    const long long mn = (long long)m * n;
    const long long o = (long long)yo * n + xo;
    const bool ring = xo == 0 || xo == n - 1 || yo == 0 || yo == m - 1;
    const long long qs = (long long)K * mn;
    for (int k = 0; k < K; ++k) {
        double* Jk = J + (long long)f * 6 * K * mn + (long long)k * mn;
        double j[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (!ring) tensor_px64(f1, f2, f, K, k, h, w, yo, xo, hy, hx, f2_f32, gray, j);
        for (int q = 0; q < 6; ++q) Jk[q * qs + o] = j[q];
    }
}

// The tensor for the float64 chained SOR, written diagonal-major: J (T, 6, K,
// D*P), pixel (r, c) at (r + c) * P + r, plus the smoothness numerator's
// constant part from the edge-padded float64 u, v (core/level_solver.py:
// 317-340): lap_u = wx ((uL - uc) + (uR - uc)) + wy ((uU - uc) + (uD - uc)),
// lap_v likewise, (T, 2, D*P).
//
// The float64 arithmetic of core/optical_flow.py:73-228 with its divisions by
// the spacings as products with their reciprocals, 1 / (sqrt(q)^2 + 1e-6) as
// 1 / (q + 1e-6), and reciprocals by Newton's iteration from the hardware
// approximation: each of these moves a value by about one rounding, far
// below what the flow is sensitive to (the tensor rounded to 48 bits moves the
// flow by 1e-8 px), at about 70 instead of 185 float64 operations per pixel
// and channel.  The warped image's own derivatives keep numpy's float32
// arithmetic exactly (f2_f32, every level below the top).  f1 is the
// reference level in float64 (K, h, w), f2 the warped level (T, K, h, w).
// One warp computes 32 consecutive rows of one diagonal, so every store is
// one contiguous run; the stencil reads go through L1.
struct TensConsts {
    double ihx2, ihy2, ihxx, ihyy;  // 1 / (2 hx), 1 / (2 hy), 1 / hx^2, 1 / hy^2
    double ihy4;                    // 1 / (4 hy) = ihy2 / 2, exact
    float h2x_f, h2y_f, hxx_f, hyy_f;
};

TensConsts tens_consts(double hy, double hx)
{
    TensConsts C;
    const double h2x = 2.0 * hx, h2y = 2.0 * hy, hxx = hx * hx, hyy = hy * hy;
    C.ihx2 = 1.0 / h2x;
    C.ihy2 = 1.0 / h2y;
    C.ihxx = 1.0 / hxx;
    C.ihyy = 1.0 / hyy;
    C.ihy4 = 0.5 * C.ihy2;
    C.h2x_f = (float)h2x;
    C.h2y_f = (float)h2y;
    C.hxx_f = (float)hxx;
    C.hyy_f = (float)hyy;
    return C;
}

__device__ __forceinline__ double drcp(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = __fma_rn(-x, y, 1.0);
    y = __fma_rn(y, e, y);
    e = __fma_rn(-x, y, 1.0);
    return __fma_rn(y, e, y);
}

// The reference level's own derivatives, the same for every frame: planes
// (4, K, h, w) of gx1 = (f1[x+1] - f1[x-1]) / (2 hx), gy1 likewise,
// fxx1 = (f1[x-1] - 2 f1 + f1[x+1]) / hx^2 and fyy1, at every pixel with the
// level's clamped neighbours, computed once per reference by kx_ref_derivs.
constexpr int kRefGx = 0, kRefGy = 1, kRefFxx = 2, kRefFyy = 3;

__device__ __forceinline__ void ref_derivs64(const double* __restrict__ a, int h, int w, int yy, int xx,
                                             const TensConsts& C, double* o)
{
    // unpadded reads at padded (yy, xx), clamped into the level
    auto A = [&](int y, int x) { return a[(long long)xclamp(y - 1, 0, h - 1) * w + xclamp(x - 1, 0, w - 1)]; };
    const double a0 = A(yy, xx);
    o[kRefGx] = dmul(dsub(A(yy, xx + 1), A(yy, xx - 1)), C.ihx2);
    o[kRefGy] = dmul(dsub(A(yy + 1, xx), A(yy - 1, xx)), C.ihy2);
    o[kRefFxx] = dmul(dadd(dsub(A(yy, xx - 1), dadd(a0, a0)), A(yy, xx + 1)), C.ihxx);
    o[kRefFyy] = dmul(dadd(dsub(A(yy - 1, xx), dadd(a0, a0)), A(yy + 1, xx)), C.ihyy);
}

// a: the reference level (h, w) of channel k in float64; rd: its derivative
// planes (plane q at rd + q * rd_ps, row-major h x w).
__device__ __forceinline__ void tensor_fast64(const double* __restrict__ a, const double* __restrict__ rd,
                                              long long rd_ps, const float* __restrict__ b, int h, int w, int yo,
                                              int xo, const TensConsts& C, int f2_f32, int gray, double* jo)
{
    // unpadded reads at padded (yy, xx), clamped into the level
    auto at = [&](int yy, int xx) { return (long long)xclamp(yy - 1, 0, h - 1) * w + xclamp(xx - 1, 0, w - 1); };
    auto A = [&](int yy, int xx) { return a[at(yy, xx)]; };
    auto Bf = [&](int yy, int xx) { return b[at(yy, xx)]; };
    auto R = [&](int q, int yy, int xx) { return rd[q * rd_ps + at(yy, xx)]; };
    auto gx2 = [&](int yy, int xx) {
        if (f2_f32) return f2d(__fdiv_rn(__fsub_rn(Bf(yy, xx + 1), Bf(yy, xx - 1)), C.h2x_f));
        return dmul(dsub(f2d(Bf(yy, xx + 1)), f2d(Bf(yy, xx - 1))), C.ihx2);
    };
    auto gy2 = [&](int yy, int xx) {
        if (f2_f32) return f2d(__fdiv_rn(__fsub_rn(Bf(yy + 1, xx), Bf(yy - 1, xx)), C.h2y_f));
        return dmul(dsub(f2d(Bf(yy + 1, xx)), f2d(Bf(yy - 1, xx))), C.ihy2);
    };
    // twice fx, fy (gx1 + gx2) at a position clamped into [1, h] x [1, w]: the halving is
    // exact, so it moves into the spacing factor of the derivative taken from them
    auto FX2 = [&](int yy, int xx) {
        yy = xclamp(yy, 1, h);
        xx = xclamp(xx, 1, w);
        return dadd(R(kRefGx, yy, xx), gx2(yy, xx));
    };
    auto FY2 = [&](int yy, int xx) {
        yy = xclamp(yy, 1, h);
        xx = xclamp(xx, 1, w);
        return dadd(R(kRefGy, yy, xx), gy2(yy, xx));
    };
    auto FT = [&](int yy, int xx) {
        yy = xclamp(yy, 1, h);
        xx = xclamp(xx, 1, w);
        return dsub(f2d(Bf(yy, xx)), A(yy, xx));
    };
    if (gray) {
        const double fxv = dmul(0.5, FX2(yo, xo)), fyv = dmul(0.5, FY2(yo, xo)), ftv = FT(yo, xo);
        jo[0] = dmul(fxv, fxv);
        jo[1] = dmul(fyv, fyv);
        jo[2] = dmul(ftv, ftv);
        jo[3] = dmul(fxv, fyv);
        jo[4] = dmul(fxv, ftv);
        jo[5] = dmul(fyv, ftv);
        return;
    }
    const double fxy = dmul(dsub(FX2(yo + 1, xo), FX2(yo - 1, xo)), C.ihy4);
    const double fxt = dmul(dsub(FT(yo, xo + 1), FT(yo, xo - 1)), C.ihx2);
    const double fyt = dmul(dsub(FT(yo + 1, xo), FT(yo - 1, xo)), C.ihy2);
    const double fxx1 = R(kRefFxx, yo, xo);
    const double fyy1 = R(kRefFyy, yo, xo);
    double fxx2, fyy2;
    if (f2_f32) {
        fxx2 = f2d(__fdiv_rn(__fadd_rn(__fsub_rn(Bf(yo, xo - 1), __fmul_rn(2.0f, Bf(yo, xo))), Bf(yo, xo + 1)),
                             C.hxx_f));
        fyy2 = f2d(__fdiv_rn(__fadd_rn(__fsub_rn(Bf(yo - 1, xo), __fmul_rn(2.0f, Bf(yo, xo))), Bf(yo + 1, xo)),
                             C.hyy_f));
    } else {
        const double b0 = f2d(Bf(yo, xo));
        fxx2 = dmul(dadd(dsub(f2d(Bf(yo, xo - 1)), dadd(b0, b0)), f2d(Bf(yo, xo + 1))), C.ihxx);
        fyy2 = dmul(dadd(dsub(f2d(Bf(yo - 1, xo)), dadd(b0, b0)), f2d(Bf(yo + 1, xo))), C.ihyy);
    }
    const double fxx = dmul(0.5, dadd(fxx1, fxx2));
    const double fyy = dmul(0.5, dadd(fyy1, fyy2));
    const double xx2 = dmul(fxx, fxx), xy2 = dmul(fxy, fxy), yy2 = dmul(fyy, fyy);
    const double reg_x = drcp(dadd(dadd(xx2, xy2), 1e-6));
    const double reg_y = drcp(dadd(dadd(xy2, yy2), 1e-6));
    const double rxx = dmul(reg_x, fxx), rxy = dmul(reg_x, fxy);  // reg_x fxx, reg_x fxy
    const double ryx = dmul(reg_y, fxy), ryy = dmul(reg_y, fyy);  // reg_y fxy, reg_y fyy
    jo[0] = __fma_rn(rxx, fxx, dmul(ryx, fxy));
    jo[1] = __fma_rn(rxy, fxy, dmul(ryy, fyy));
    jo[2] = __fma_rn(dmul(reg_x, fxt), fxt, dmul(dmul(reg_y, fyt), fyt));
    jo[3] = __fma_rn(rxx, fxy, dmul(ryx, fyy));
    jo[4] = __fma_rn(rxx, fxt, dmul(ryx, fyt));
    jo[5] = __fma_rn(rxy, fxt, dmul(ryy, fyt));
}

__global__ void kx_ref_derivs(const double* __restrict__ f1, int K, int h, int w, TensConsts C, double* __restrict__ rd)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    const int k = blockIdx.z;
    if (c >= w) return;
    const long long hw = (long long)h * w;
    double o[4];
    ref_derivs64(f1 + k * hw, h, w, r + 1, c + 1, C, o);
#pragma unroll
    for (int q = 0; q < 4; ++q) rd[((long long)q * K + k) * hw + (long long)r * w + c] = o[q];
}

cudaError_t launch_x_ref_derivs(const double* f1, int K, int h, int w, double hy, double hx, double* rd,
                                cudaStream_t st)
{
    dim3 blk(128), grd((w + 127) / 128, h, K);
    kx_ref_derivs<<<grd, blk, 0, st>>>(f1, K, h, w, tens_consts(hy, hx), rd);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) kx_tensor_diag(const double* __restrict__ f1, const double* __restrict__ rd,
                                                      const float* __restrict__ f1f,
                                                      const float* __restrict__ f2, int K, int h, int w, TensConsts C,
                                                      double hy, double hx, int f2_f32, int gray,
                                                      double* __restrict__ J, long long J_fs, DiagGeom g,
                                                      const double* __restrict__ u, const double* __restrict__ v,
                                                      long long uv_fs, double wx, double wy, double* __restrict__ lap,
                                                      long long lap_fs)
{
    const int nstrip = g.P >> 5;
    const long long wid = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (wid >= (long long)g.D * nstrip) return;
    const int d = (int)(wid / nstrip);
    const int r = (int)(wid - (long long)d * nstrip) * 32 + (threadIdx.x & 31);
    const int c = d - r;
    if (r >= h || c < 0 || c >= w) return;
    const int f = blockIdx.y;
    const long long plane = (long long)g.D * g.P;
    const long long di = (long long)d * g.P + r;
    const long long hw = (long long)h * w;
    double* Jf = J + f * J_fs;
    for (int k = 0; k < K; ++k) {
        double j[6];
        if (gray == 2)  // census: the reference-order arithmetic of kx_tensor
            tensor_px64(f1f, f2, f, K, k, h, w, r + 1, c + 1, hy, hx, f2_f32, 2, j);
        else
            tensor_fast64(f1 + k * hw, rd + k * hw, K * hw, f2 + ((long long)f * K + k) * hw, h, w, r + 1, c + 1, C,
                          f2_f32, gray, j);
        // the cross terms doubled (exact), as the solver's data residual uses them, and
        // J33 with the residual's offset 1e-5 added
#pragma unroll
        for (int q = 0; q < 6; ++q)
            Jf[((long long)q * K + k) * plane + di] = q < 2 ? j[q] : (q == 2 ? dadd(j[2], 0.00001) : dadd(j[q], j[q]));
    }
    const long long n = w + 2;
    const double* uf = u + f * uv_fs;
    const double* vf = v + f * uv_fs;
    const long long o = (long long)(r + 1) * n + c + 1;
    const double uc = uf[o], vc = vf[o];
    const double lu = __fma_rn(wx, dadd(dsub(uf[o - 1], uc), dsub(uf[o + 1], uc)),
                               dmul(wy, dadd(dsub(uf[o - n], uc), dsub(uf[o + n], uc))));
    const double lv = __fma_rn(wx, dadd(dsub(vf[o - 1], vc), dsub(vf[o + 1], vc)),
                               dmul(wy, dadd(dsub(vf[o - n], vc), dsub(vf[o + n], vc))));
    lap[f * lap_fs + di] = lu;
    lap[f * lap_fs + plane + di] = lv;
}

cudaError_t launch_x_tensor(const float* f1, const float* f2, int n_frames, int K, int h, int w, double hy, double hx,
                            int f2_f32, int gray, double* J, cudaStream_t st)
{
    dim3 blk(128), grd((w + 2 + 127) / 128, h + 2, n_frames);
    kx_tensor<<<grd, blk, 0, st>>>(f1, f2, K, h, w, hy, hx, f2_f32, gray, J);
    return cudaGetLastError();
}

cudaError_t launch_x_tensor_diag(const double* f1, const double* rd, const float* f1f, const float* f2, int n_frames,
                                 int K, int h, int w, double hy, double hx, int f2_f32, int gray, double* J,
                                 long long J_fs, DiagGeom g, const double* u, const double* v, long long uv_fs,
                                 double wx, double wy, double* lap, long long lap_fs, cudaStream_t st)
{
    const TensConsts C = tens_consts(hy, hx);
    const long long warps = (long long)g.D * (g.P >> 5);
    if ((warps + 7) / 8 > 0x7fffffffLL || n_frames > 65535) return cudaErrorInvalidValue;
    dim3 grd((unsigned)((warps + 7) / 8), n_frames);
    kx_tensor_diag<<<grd, 256, 0, st>>>(f1, rd, f1f, f2, K, h, w, C, hy, hx, f2_f32, gray, J, J_fs, g, u, v, uv_fs,
                                        wx, wy, lap, lap_fs);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// compute_flow (core/level_solver.py:158-369) in its own order and arithmetic,
// all iterations in one launch.  One CTA per frame, threads over rows; the
// exact lexicographic order is kept by the wavefront schedule of the FP32
// solver (pixel (r, c) of iteration t at step r + c + 2t), here on global
// memory so that any number of iterations is pipelined.  The psi update of a
// tick iteration is pixel-local, so it is applied to each pixel just before
// its own update, from its own (iteration t-1) du, dv -- the same values the
// reference's full-array psi pass reads.  __syncthreads orders the global
// stores of one step before the loads of the next within the CTA.
// J: (T, 6, K, m*n); W: (K, m*n) shared; u, v: (T, m*n) (frame stride uv_fs);
// du, dv: (T, m*n); wp: (T, K, m*n) scratch holding weight * psi.
// ---------------------------------------------------------------------------
struct XAData { double a[kMaxK]; };

// compute_flow_gnc (core/level_solver.py:408-446): with a stage weight beta in
// [0, 1) (beta < 0: no GNC) an exponent a in (0, 1) gives (1 - beta) + beta * robust.
__device__ __forceinline__ double gnc_mix(double robust, double a, double beta)
{
    if (beta >= 0.0 && beta < 1.0 && a > 0.0 && a < 1.0) return dadd(dsub(1.0, beta), dmul(beta, robust));
    return robust;
}

// set_boundary_2d (core/level_solver.py:46-67) at the start of the last
// iteration leaves every border cell of du, dv holding, at clamped
// coordinates, the interior value of that moment: the border-adjacent pixel
// (r, c) writes its pre-update value to the cells that clamp to it.  The
// sweep itself never reads the border (the Neumann copy is the pixel's own
// value), so only what follows the solve sees it.
__device__ __forceinline__ void ring_snapshot(double* du, double* dv, int r, int c, int h, int w, double duc,
                                              double dvc)
{
    const long long n = w + 2;
    const int ys[2] = {r == 0 ? 0 : -1, r == h - 1 ? h + 1 : -1};
    const int xs[2] = {c == 0 ? 0 : -1, c == w - 1 ? w + 1 : -1};
    for (int a = 0; a < 2; ++a) {
        if (ys[a] < 0) continue;
        const long long q = (long long)ys[a] * n + c + 1;
        du[q] = duc;
        dv[q] = dvc;
        for (int b = 0; b < 2; ++b) {
            if (xs[b] < 0) continue;
            du[(long long)ys[a] * n + xs[b]] = duc;
            dv[(long long)ys[a] * n + xs[b]] = dvc;
        }
    }
    for (int b = 0; b < 2; ++b) {
        if (xs[b] < 0) continue;
        const long long q = (long long)(r + 1) * n + xs[b];
        du[q] = duc;
        dv[q] = dvc;
    }
}

__global__ void kx_sor(const double* __restrict__ J, const double* __restrict__ W, const double* __restrict__ u,
                       const double* __restrict__ v, long long uv_fs, double* du_g, double* dv_g, double* wp_g,
                       int K, int h, int w, double alpha_x, double alpha_y, double hx, double hy, int iterations,
                       int update_lag, XAData ad, double omega, double gnc_beta)
{
    const int f = blockIdx.x;
    const int n = w + 2, m = h + 2;
    const long long mn = (long long)m * n;
    const double* Jf = J + (long long)f * 6 * K * mn;
    const double* uf = u + f * uv_fs;
    const double* vf = v + f * uv_fs;
    double* du = du_g + (long long)f * mn;
    double* dv = dv_g + (long long)f * mn;
    double* wp = wp_g + (long long)f * K * mn;
    const long long qs = (long long)K * mn;
    for (long long i = threadIdx.x; i < mn; i += blockDim.x) {
        du[i] = 0.0;
        dv[i] = 0.0;
        for (int k = 0; k < K; ++k) wp[(long long)k * mn + i] = W[(long long)k * mn + i];  // psi = 1
    }
    __syncthreads();
    const double tx = ddiv(alpha_x, dmul(hx, hx));
    const double ty = ddiv(alpha_y, dmul(hy, hy));
    const double one_m_omega = dsub(1.0, omega);
    const int nsteps = (h - 1) + (w - 1) + 2 * (iterations - 1) + 1;
    for (int s = 0; s < nsteps; ++s) {
        for (int r = threadIdx.x; r < h; r += blockDim.x) {
            // the iterations whose column s - r - 2t lies in [0, w): t from ceil((s - r - w + 1) / 2)
            // to floor((s - r) / 2), without visiting the others
            const int sr = s - r;
            if (sr < 0) continue;
            const int t_lo = sr >= w ? (sr - w + 2) / 2 : 0;
            const int t_hi = min(iterations - 1, sr / 2);
            for (int t = t_lo; t <= t_hi; ++t) {
                const int c = sr - 2 * t;
                const long long o = (long long)(r + 1) * n + (c + 1);
                const double duc = du[o], dvc = dv[o];
                if (t == iterations - 1 && (r == 0 || r == h - 1 || c == 0 || c == w - 1))
                    ring_snapshot(du, dv, r, c, h, w, duc, dvc);
                if ((t + 1) % update_lag == 0) {
                    // core/level_solver.py:230-246 (J23*dv appears twice, as in the reference)
                    for (int k = 0; k < K; ++k) {
                        const long long ok = (long long)k * mn + o;
                        double val = dmul(dmul(Jf[ok], duc), duc);
                        val = dadd(val, dmul(dmul(Jf[qs + ok], dvc), dvc));
                        val = dadd(val, dmul(Jf[5 * qs + ok], dvc));
                        val = dadd(val, dmul(dmul(dmul(2.0, Jf[3 * qs + ok]), duc), dvc));
                        val = dadd(val, dmul(dmul(2.0, Jf[4 * qs + ok]), duc));
                        val = dadd(val, dmul(Jf[5 * qs + ok], dvc));
                        val = dadd(val, Jf[2 * qs + ok]);
                        if (val < 0.0) val = 0.0;
                        const double psi =
                            gnc_mix(dmul(ad.a[k], pow(dadd(val, 0.00001), dsub(ad.a[k], 1.0))), ad.a[k], gnc_beta);
                        wp[ok] = dmul(W[ok], psi);
                    }
                }
                // neighbours; across the level border the Neumann copy equals the pixel's own old value
                const double duL = c > 0 ? du[o - 1] : duc, dvL = c > 0 ? dv[o - 1] : dvc;
                const double duR = c < w - 1 ? du[o + 1] : duc, dvR = c < w - 1 ? dv[o + 1] : dvc;
                const double duD = r < h - 1 ? du[o + n] : duc, dvD = r < h - 1 ? dv[o + n] : dvc;
                const double duU = r > 0 ? du[o - n] : duc, dvU = r > 0 ? dv[o - n] : dvc;
                const double uc = uf[o], vc = vf[o];
                double num_u = 0.0, num_v = 0.0, den_u = 0.0, den_v = 0.0;
                // left, right, down, up (core/level_solver.py:318-340)
                num_u = dadd(num_u, dmul(tx, dsub(dadd(uf[o - 1], duL), uc)));
                num_v = dadd(num_v, dmul(tx, dsub(dadd(vf[o - 1], dvL), vc)));
                den_u = dadd(den_u, tx);
                den_v = dadd(den_v, tx);
                num_u = dadd(num_u, dmul(tx, dsub(dadd(uf[o + 1], duR), uc)));
                num_v = dadd(num_v, dmul(tx, dsub(dadd(vf[o + 1], dvR), vc)));
                den_u = dadd(den_u, tx);
                den_v = dadd(den_v, tx);
                num_u = dadd(num_u, dmul(ty, dsub(dadd(uf[o + n], duD), uc)));
                num_v = dadd(num_v, dmul(ty, dsub(dadd(vf[o + n], dvD), vc)));
                den_u = dadd(den_u, ty);
                den_v = dadd(den_v, ty);
                num_u = dadd(num_u, dmul(ty, dsub(dadd(uf[o - n], duU), uc)));
                num_v = dadd(num_v, dmul(ty, dsub(dadd(vf[o - n], dvU), vc)));
                den_u = dadd(den_u, ty);
                den_v = dadd(den_v, ty);
                for (int k = 0; k < K; ++k) {
                    const long long ok = (long long)k * mn + o;
                    const double wpk = wp[ok];
                    num_u = dsub(num_u, dmul(wpk, dadd(Jf[4 * qs + ok], dmul(Jf[3 * qs + ok], dvc))));
                    den_u = dadd(den_u, dmul(wpk, Jf[ok]));
                    den_v = dadd(den_v, dmul(wpk, Jf[qs + ok]));
                }
                const double du_kp1 = den_u != 0.0 ? ddiv(num_u, den_u) : 0.0;
                const double dun = dadd(dmul(one_m_omega, duc), dmul(omega, du_kp1));
                double num_v2 = num_v;
                for (int k = 0; k < K; ++k) {
                    const long long ok = (long long)k * mn + o;
                    num_v2 = dsub(num_v2, dmul(wp[ok], dadd(Jf[5 * qs + ok], dmul(Jf[3 * qs + ok], dun))));
                }
                const double dv_kp1 = den_v != 0.0 ? ddiv(num_v2, den_v) : 0.0;
                const double dvn = dadd(dmul(one_m_omega, dvc), dmul(omega, dv_kp1));
                du[o] = dun;
                dv[o] = dvn;
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_x_sor(const double* J, const double* W, const double* u, const double* v, long long uv_fs,
                         double* du, double* dv, double* wp, int n_frames, int K, int h, int w, double alpha_x,
                         double alpha_y, double hx, double hy, int iterations, int update_lag,
                         const double* a_data, double omega, double gnc_beta, cudaStream_t st)
{
    XAData ad;
    for (int k = 0; k < kMaxK; ++k) ad.a[k] = k < K ? a_data[k] : 0.0;
    const int threads = h >= 512 ? 512 : ((h + 31) / 32) * 32;
    kx_sor<<<n_frames, threads, 0, st>>>(J, W, u, v, uv_fs, du, dv, wp, K, h, w, alpha_x, alpha_y, hx, hy,
                                         iterations, update_lag, ad, omega, gnc_beta);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// a_smooth != 1 (core/level_solver.py:69-155, 229-255, 309-340).  The
// smoothness weights psi_s need every pixel's u + du at the start of a tick
// iteration, so the wavefront is cut at the ticks: kx_smooth_tick computes the
// data weights W psi and psi_s over the whole padded grid, kx_sor_range runs
// the iterations up to the next tick.  psi_s reads the border of du, dv as
// set_boundary_2d last left it: at the start of the previous iteration, i.e.
// the interior values then, taken at clamped coordinates.  kx_sor_range
// snapshots every pixel's value before its update in the range's last
// iteration for that purpose.
// ---------------------------------------------------------------------------
__global__ void kx_smooth_init(const double* __restrict__ W, double* __restrict__ wp, double* __restrict__ psi_s,
                               double* __restrict__ snap, int K, long long mn)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long f = blockIdx.y;
    if (i >= mn) return;
    for (int k = 0; k < K; ++k) wp[(f * K + k) * mn + i] = W[(long long)k * mn + i];
    psi_s[f * mn + i] = 1.0;
    snap[f * 2 * mn + i] = 0.0;
    snap[f * 2 * mn + mn + i] = 0.0;
}

__global__ void kx_smooth_tick(const double* __restrict__ J, const double* __restrict__ W,
                               const double* __restrict__ u, const double* __restrict__ v, long long uv_fs,
                               const double* __restrict__ du_g, const double* __restrict__ dv_g,
                               const double* __restrict__ snap, double* __restrict__ wp_g, double* __restrict__ psi_g,
                               int K, int h, int w, double hx, double hy, XAData ad, double a_s, double gnc_beta)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // column of the padded grid
    const int j = blockIdx.y;                              // row of the padded grid
    const long long f = blockIdx.z;
    const int n = w + 2, m = h + 2;
    if (i >= n) return;
    const long long mn = (long long)m * n, o = (long long)j * n + i;
    const double* du = du_g + f * mn;
    const double* dv = dv_g + f * mn;
    const double* sn = snap + f * 2 * mn;
    const double* uf = u + f * uv_fs;
    const double* vf = v + f * uv_fs;
    const bool interior = j >= 1 && j <= m - 2 && i >= 1 && i <= n - 2;
    if (interior) {
        // data weights (core/level_solver.py:230-246), as kx_sor computes them
        const double duc = du[o], dvc = dv[o];
        const double* Jf = J + f * 6 * K * mn;
        const long long qs = (long long)K * mn;
        for (int k = 0; k < K; ++k) {
            const long long ok = (long long)k * mn + o;
            double val = dmul(dmul(Jf[ok], duc), duc);
            val = dadd(val, dmul(dmul(Jf[qs + ok], dvc), dvc));
            val = dadd(val, dmul(Jf[5 * qs + ok], dvc));
            val = dadd(val, dmul(dmul(dmul(2.0, Jf[3 * qs + ok]), duc), dvc));
            val = dadd(val, dmul(dmul(2.0, Jf[4 * qs + ok]), duc));
            val = dadd(val, dmul(Jf[5 * qs + ok], dvc));
            val = dadd(val, Jf[2 * qs + ok]);
            if (val < 0.0) val = 0.0;
            const double psi =
                gnc_mix(dmul(ad.a[k], pow(dadd(val, 0.00001), dsub(ad.a[k], 1.0))), ad.a[k], gnc_beta);
            wp_g[(f * K + k) * mn + o] = dmul(W[ok], psi);
        }
    }
    // u + du at padded (jj, ii): the interior now, the border as set_boundary_2d left it
    auto full = [&](int jj, int ii, int plane) {
        const long long q = (long long)jj * n + ii;
        const bool in = jj >= 1 && jj <= m - 2 && ii >= 1 && ii <= n - 2;
        double d;
        if (in)
            d = plane ? dv[q] : du[q];
        else
            d = sn[(long long)plane * mn + (long long)xclamp(jj, 1, m - 2) * n + xclamp(ii, 1, n - 2)];
        return dadd(plane ? vf[q] : uf[q], d);
    };
    double ux = 0.0, vx = 0.0, uy = 0.0, vy = 0.0;
    if (n > 1) {
        if (i == 0) {
            ux = ddiv(dsub(full(j, i + 1, 0), full(j, i, 0)), hx);
            vx = ddiv(dsub(full(j, i + 1, 1), full(j, i, 1)), hx);
        } else if (i == n - 1) {
            ux = ddiv(dsub(full(j, i, 0), full(j, i - 1, 0)), hx);
            vx = ddiv(dsub(full(j, i, 1), full(j, i - 1, 1)), hx);
        } else {
            ux = ddiv(dsub(full(j, i + 1, 0), full(j, i - 1, 0)), dmul(2.0, hx));
            vx = ddiv(dsub(full(j, i + 1, 1), full(j, i - 1, 1)), dmul(2.0, hx));
        }
    }
    if (m > 1) {
        if (j == 0) {
            uy = ddiv(dsub(full(j + 1, i, 0), full(j, i, 0)), hy);
            vy = ddiv(dsub(full(j + 1, i, 1), full(j, i, 1)), hy);
        } else if (j == m - 1) {
            uy = ddiv(dsub(full(j, i, 0), full(j - 1, i, 0)), hy);
            vy = ddiv(dsub(full(j, i, 1), full(j - 1, i, 1)), hy);
        } else {
            uy = ddiv(dsub(full(j + 1, i, 0), full(j - 1, i, 0)), dmul(2.0, hy));
            vy = ddiv(dsub(full(j + 1, i, 1), full(j - 1, i, 1)), dmul(2.0, hy));
        }
    }
    double tmp = dadd(dadd(dadd(dmul(ux, ux), dmul(uy, uy)), dmul(vx, vx)), dmul(vy, vy));
    if (tmp < 0.0) tmp = 0.0;
    psi_g[f * mn + o] = gnc_mix(dmul(a_s, pow(dadd(tmp, 0.00001), dsub(a_s, 1.0))), a_s, gnc_beta);
}

// Iterations [t0, t1) of the lexicographic SOR as one wavefront (pixel (r, c)
// of iteration t at step r + c + 2 (t - t0)) with the weights of the last tick
// and the smoothness weights 0.5 (psi_s[c] + psi_s[n]) alpha / h^2.
__global__ void kx_sor_range(const double* __restrict__ J, const double* __restrict__ u,
                             const double* __restrict__ v, long long uv_fs, double* du_g, double* dv_g,
                             const double* __restrict__ wp_g, const double* __restrict__ psi_g,
                             double* __restrict__ snap, int K, int h, int w, double alpha_x, double alpha_y, double hx,
                             double hy, int t0, int t1, double omega)
{
    const int f = blockIdx.x;
    const int n = w + 2, m = h + 2;
    const long long mn = (long long)m * n;
    const double* Jf = J + (long long)f * 6 * K * mn;
    const double* uf = u + f * uv_fs;
    const double* vf = v + f * uv_fs;
    double* du = du_g + (long long)f * mn;
    double* dv = dv_g + (long long)f * mn;
    const double* wp = wp_g + (long long)f * K * mn;
    const double* ps = psi_g + (long long)f * mn;
    double* sn = snap + (long long)f * 2 * mn;
    const long long qs = (long long)K * mn;
    const double ax = ddiv(alpha_x, dmul(hx, hx));
    const double ay = ddiv(alpha_y, dmul(hy, hy));
    const double one_m_omega = dsub(1.0, omega);
    const int nit = t1 - t0;
    const int nsteps = (h - 1) + (w - 1) + 2 * (nit - 1) + 1;
    for (int s = 0; s < nsteps; ++s) {
        for (int r = threadIdx.x; r < h; r += blockDim.x) {
            const int sr = s - r;
            if (sr < 0) continue;
            const int t_lo = sr >= w ? (sr - w + 2) / 2 : 0;
            const int t_hi = min(nit - 1, sr / 2);
            for (int tl = t_lo; tl <= t_hi; ++tl) {
                const int c = sr - 2 * tl;
                const long long o = (long long)(r + 1) * n + (c + 1);
                const double duc = du[o], dvc = dv[o];
                if (tl == nit - 1) {
                    sn[o] = duc;
                    sn[mn + o] = dvc;
                    if (r == 0 || r == h - 1 || c == 0 || c == w - 1) ring_snapshot(du, dv, r, c, h, w, duc, dvc);
                }
                const double duL = c > 0 ? du[o - 1] : duc, dvL = c > 0 ? dv[o - 1] : dvc;
                const double duR = c < w - 1 ? du[o + 1] : duc, dvR = c < w - 1 ? dv[o + 1] : dvc;
                const double duD = r < h - 1 ? du[o + n] : duc, dvD = r < h - 1 ? dv[o + n] : dvc;
                const double duU = r > 0 ? du[o - n] : duc, dvU = r > 0 ? dv[o - n] : dvc;
                const double uc = uf[o], vc = vf[o], pc = ps[o];
                double num_u = 0.0, num_v = 0.0, den_u = 0.0, den_v = 0.0, t;
                // left, right, down, up (core/level_solver.py:272-307)
                t = dmul(dmul(0.5, dadd(pc, ps[o - 1])), ax);
                num_u = dadd(num_u, dmul(t, dsub(dadd(uf[o - 1], duL), uc)));
                num_v = dadd(num_v, dmul(t, dsub(dadd(vf[o - 1], dvL), vc)));
                den_u = dadd(den_u, t);
                den_v = dadd(den_v, t);
                t = dmul(dmul(0.5, dadd(pc, ps[o + 1])), ax);
                num_u = dadd(num_u, dmul(t, dsub(dadd(uf[o + 1], duR), uc)));
                num_v = dadd(num_v, dmul(t, dsub(dadd(vf[o + 1], dvR), vc)));
                den_u = dadd(den_u, t);
                den_v = dadd(den_v, t);
                t = dmul(dmul(0.5, dadd(pc, ps[o + n])), ay);
                num_u = dadd(num_u, dmul(t, dsub(dadd(uf[o + n], duD), uc)));
                num_v = dadd(num_v, dmul(t, dsub(dadd(vf[o + n], dvD), vc)));
                den_u = dadd(den_u, t);
                den_v = dadd(den_v, t);
                t = dmul(dmul(0.5, dadd(pc, ps[o - n])), ay);
                num_u = dadd(num_u, dmul(t, dsub(dadd(uf[o - n], duU), uc)));
                num_v = dadd(num_v, dmul(t, dsub(dadd(vf[o - n], dvU), vc)));
                den_u = dadd(den_u, t);
                den_v = dadd(den_v, t);
                for (int k = 0; k < K; ++k) {
                    const long long ok = (long long)k * mn + o;
                    const double wpk = wp[ok];
                    num_u = dsub(num_u, dmul(wpk, dadd(Jf[4 * qs + ok], dmul(Jf[3 * qs + ok], dvc))));
                    den_u = dadd(den_u, dmul(wpk, Jf[ok]));
                    den_v = dadd(den_v, dmul(wpk, Jf[qs + ok]));
                }
                const double du_kp1 = den_u != 0.0 ? ddiv(num_u, den_u) : 0.0;
                const double dun = dadd(dmul(one_m_omega, duc), dmul(omega, du_kp1));
                double num_v2 = num_v;
                for (int k = 0; k < K; ++k) {
                    const long long ok = (long long)k * mn + o;
                    num_v2 = dsub(num_v2, dmul(wp[ok], dadd(Jf[5 * qs + ok], dmul(Jf[3 * qs + ok], dun))));
                }
                const double dv_kp1 = den_v != 0.0 ? ddiv(num_v2, den_v) : 0.0;
                const double dvn = dadd(dmul(one_m_omega, dvc), dmul(omega, dv_kp1));
                du[o] = dun;
                dv[o] = dvn;
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_x_sor_smooth(const double* J, const double* W, const double* u, const double* v, long long uv_fs,
                                double* du, double* dv, double* wp, double* psi_s, double* snap, int n_frames, int K,
                                int h, int w, double alpha_x, double alpha_y, double hx, double hy, int iterations,
                                int update_lag, const double* a_data, double a_smooth, double omega, double gnc_beta,
                                cudaStream_t st, long long* launches)
{
    XAData ad;
    for (int k = 0; k < kMaxK; ++k) ad.a[k] = k < K ? a_data[k] : 0.0;
    const long long mn = (long long)(h + 2) * (w + 2);
    cudaError_t e = cudaMemsetAsync(du, 0, sizeof(double) * n_frames * mn, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dv, 0, sizeof(double) * n_frames * mn, st);
    if (e != cudaSuccess) return e;
    kx_smooth_init<<<dim3((unsigned)((mn + 255) / 256), (unsigned)n_frames), 256, 0, st>>>(W, wp, psi_s, snap, K, mn);
    ++*launches;
    const int threads = h >= 512 ? 512 : ((h + 31) / 32) * 32;
    int t = 0;
    while (t < iterations) {
        if ((t + 1) % update_lag == 0) {
            kx_smooth_tick<<<dim3((unsigned)((w + 2 + 127) / 128), (unsigned)(h + 2), (unsigned)n_frames), 128, 0, st>>>(
                J, W, u, v, uv_fs, du, dv, snap, wp, psi_s, K, h, w, hx, hy, ad, a_smooth, gnc_beta);
            ++*launches;
        }
        int t1 = t + 1;
        while (t1 < iterations && (t1 + 1) % update_lag != 0) ++t1;
        kx_sor_range<<<n_frames, threads, 0, st>>>(J, u, v, uv_fs, du, dv, wp, psi_s, snap, K, h, w, alpha_x, alpha_y,
                                                   hx, hy, t, t1, omega);
        ++*launches;
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        t = t1;
    }
    return cudaSuccess;
}

__global__ void kx_to_double(const float* __restrict__ src, long long n, double* __restrict__ dst)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (double)src[i];
}

cudaError_t launch_x_to_double(const float* src, long long n, double* dst, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    kx_to_double<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, n, dst);
    return cudaGetLastError();
}

// Padded (K, m*n) planes (the interior at (1, 1)) to diagonal-major (K, D*P);
// with scale set, also the planes times scale[k] at dst + K*D*P.
struct ChannelScale {
    double s[kMaxK];
};

__global__ void kx_pad_to_diag(const double* __restrict__ src, int K, int h, int w, DiagGeom g, double* __restrict__ dst,
                               ChannelScale sc, int scaled)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    const int k = blockIdx.z;
    if (c >= w || k >= K) return;
    const long long n = w + 2, mn = (long long)(h + 2) * n;
    const long long plane = (long long)g.D * g.P, di = diag_index(g, r, c);
    const double v = src[k * mn + (long long)(r + 1) * n + c + 1];
    dst[k * plane + di] = v;
    if (scaled) dst[(K + k) * plane + di] = dmul(v, sc.s[k]);
}

cudaError_t launch_x_pad_to_diag(const double* src, int K, int h, int w, DiagGeom g, double* dst, cudaStream_t st,
                                 const double* scale)
{
    if (K < 1 || K > kMaxK) return cudaErrorInvalidValue;
    ChannelScale sc = {};
    if (scale)
        for (int k = 0; k < K; ++k) sc.s[k] = scale[k];
    dim3 blk(128), grd((w + 127) / 128, h, K);
    kx_pad_to_diag<<<grd, blk, 0, st>>>(src, K, h, w, g, dst, sc, scale ? 1 : 0);
    return cudaGetLastError();
}

__global__ void kx_to_float(const double* __restrict__ src, long long n, float* __restrict__ dst)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

cudaError_t launch_x_to_float(const double* src, long long n, float* dst, cudaStream_t st)
{
    kx_to_float<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, n, dst);
    return cudaGetLastError();
}

// n_arrays arrays of (mn, K) channel-last doubles -> (n_arrays, K, mn) planes
__global__ void kx_hwk_to_planes(const double* __restrict__ src, long long mn, int K, double* __restrict__ dst)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long a = blockIdx.y;
    if (i >= mn) return;
    for (int k = 0; k < K; ++k) dst[(a * K + k) * mn + i] = src[(a * mn + i) * K + k];
}

cudaError_t launch_x_hwk_to_planes(const double* src, int n_arrays, long long mn, int K, double* dst, cudaStream_t st)
{
    kx_hwk_to_planes<<<dim3((unsigned)((mn + 255) / 256), (unsigned)n_arrays), 256, 0, st>>>(src, mn, K, dst);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Median (scipy "mirror", exact selection) and accumulate in float64
// (core/optical_flow.py:607-611).  du, dv, u, v: padded (m, n) planes; output
// u + du, v + dv interiors with strides (frame, row, col) in elements.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dswap(double& x, double& y)
{
    const double lo = fmin(x, y), hi = fmax(x, y);
    x = lo;
    y = hi;
}

__device__ __forceinline__ void uswap(unsigned& x, unsigned& y)
{
    const unsigned lo = min(x, y), hi = max(x, y);
    x = lo;
    y = hi;
}

// The 13th smallest of 25 values: forgetful selection (keep 14 candidates,
// repeatedly drop the minimum and the maximum and admit the next value; the
// middle of the last three is the median).
template <class T>
__device__ __forceinline__ T median25_net(const T v[25])
{
    T t[14];
#pragma unroll
    for (int i = 0; i < 14; ++i) t[i] = v[i];
#pragma unroll
    for (int round = 0; round < 11; ++round) {
        const int lo = round;
#pragma unroll
        for (int i = lo + 1; i < 14; ++i) {
            if constexpr (sizeof(T) == 8) dswap(t[lo], t[i]);
            else uswap(t[lo], t[i]);
        }
#pragma unroll
        for (int i = lo + 1; i < 13; ++i) {
            if constexpr (sizeof(T) == 8) dswap(t[i], t[13]);
            else uswap(t[i], t[13]);
        }
        t[13] = v[14 + round];
    }
    if constexpr (sizeof(T) == 8) {
        dswap(t[11], t[12]);
        dswap(t[12], t[13]);
        dswap(t[11], t[12]);
    } else {
        uswap(t[11], t[12]);
        uswap(t[12], t[13]);
        uswap(t[11], t[12]);
    }
    return t[12];
}

__device__ double median25d(double v[25]) { return median25_net<double>(v); }

// The same median with the comparisons on the float32 and integer pipes.  The
// high word of a double (sign, exponent, top 20 bits of the fraction), read as
// a float, orders like the double itself as long as it is a finite float
// (|x| < 2^1017): both are sign-magnitude encodings with the magnitude bits in
// significance order.  The 13th smallest key km is found by the selection
// network on floats; if exactly one value carries it, that value is the
// median.  Several values carry km when they agree in their top 20 fraction
// bits, which smooth flow fields make common; median25_tie then decides from
// the low words.  A key that is not a finite float, or km = 0 (the keys of +0
// and -0 compare equal with different high words), leaves the decision to
// median25d on the doubles.
__device__ __forceinline__ float hikey(double x) { return __int_as_float(__double2hiint(x)); }

// The median of 25 doubles (get(i), i < 25) whose 13th smallest key km (finite,
// non-zero) is carried by eq > 1 of them, nlt keys being smaller.  A finite
// non-zero float equals only its own bit pattern, so the values that carry km
// share their high word and with it their sign, and their low words order them:
// ascending for a positive km, descending for a negative one.  With the low
// word complemented for a negative km, the tie key t (0 below km, the low word
// at km, ~0 above) is non-decreasing in the values' order, so the 13th smallest
// t is the median's low word.  It is the smallest tied t when the median is the
// first tied value in order (r = 12 - nlt = 0), the largest when it is the last
// (r = eq - 1: every two-way tie is one of the two), and otherwise the 25-value
// selection on the tie keys, on the integer pipe.
template <class Get>
__device__ __forceinline__ double median25_tie(Get get, float km, int nlt, int eq)
{
    const unsigned s = (__float_as_uint(km) >> 31) ? 0xffffffffu : 0u;
    const int r = 12 - nlt;
    unsigned tm;
    if (r == 0 || r == eq - 1) {
        unsigned tmin = 0xffffffffu, tmax = 0u;
#pragma unroll
        for (int i = 0; i < 25; ++i) {
            const double x = get(i);
            if (hikey(x) == km) {
                const unsigned t = (unsigned)__double2loint(x) ^ s;
                tmin = min(tmin, t);
                tmax = max(tmax, t);
            }
        }
        tm = r == 0 ? tmin : tmax;
    } else {
        unsigned t[25];
#pragma unroll
        for (int i = 0; i < 25; ++i) {
            const double x = get(i);
            const float k = hikey(x);
            t[i] = k < km ? 0u : (k > km ? 0xffffffffu : (unsigned)__double2loint(x) ^ s);
        }
        tm = median25_net<unsigned>(t);
    }
    return __hiloint2double(__float_as_int(km), (int)(tm ^ s));
}

__device__ __forceinline__ void fswap(float& x, float& y)
{
    const float lo = fminf(x, y), hi = fmaxf(x, y);
    x = lo;
    y = hi;
}

__device__ double median25_keys(double v[25])
{
    float t[14];
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 14; ++i) {
        t[i] = hikey(v[i]);
        finite = finite && fabsf(t[i]) <= 3.402823466e38f;
    }
#pragma unroll
    for (int round = 0; round < 11; ++round) {
        const int lo = round;
#pragma unroll
        for (int i = lo + 1; i < 14; ++i) fswap(t[lo], t[i]);
#pragma unroll
        for (int i = lo + 1; i < 13; ++i) fswap(t[i], t[13]);
        t[13] = hikey(v[14 + round]);
        finite = finite && fabsf(t[13]) <= 3.402823466e38f;
    }
    fswap(t[11], t[12]);
    fswap(t[12], t[13]);
    fswap(t[11], t[12]);
    const float m = t[12];
    int eq = 0, nlt = 0;
    double pick = 0.0;
#pragma unroll
    for (int i = 0; i < 25; ++i) {
        const float k = hikey(v[i]);
        nlt += k < m;
        if (k == m) {
            ++eq;
            pick = v[i];
        }
    }
    if (finite && eq == 1) return pick;
    if (finite && m != 0.0f) return median25_tie([&](int i) { return v[i]; }, m, nlt, eq);
    return median25d(v);
}

// Median + accumulate on float64 du, dv (the interiors of the padded level
// planes: du[y * s_rs + x], frames s_fs apart), exact like median25_keys: a
// 32 x 16 output tile with its mirrored 2-pixel halo is staged in shared
// memory as the doubles and their float keys (high words); each thread takes
// two vertically adjacent pixels, whose windows share four of their five rows,
// and median25_pair finds both windows' 13th smallest keys on the float pipe.
// A key carried by exactly one value of its window names the median; several
// values carrying it go to median25_tie (integer pipe), and a key that is not a
// finite float, or a zero key, to median25d.  Writes u + median(du) (u, v the
// padded planes, frames uv_fs apart), or the median itself when u is null.
// Needs h, w >= 3 when do_median.
constexpr int kXMedTx = 32, kXMedTy = 8, kXMedRows = 2 * kXMedTy;

__device__ __forceinline__ int mirror_x(int i, int n)
{
    if (i < 0) i = -i;
    if (i >= n) i = 2 * (n - 1) - i;
    return i;
}

__global__ void __launch_bounds__(kXMedTx * kXMedTy) kx_median_rm(const double* __restrict__ du,
                                                                 const double* __restrict__ dv, long long s_fs,
                                                                 long long s_rs, const double* __restrict__ u,
                                                                 const double* __restrict__ v, long long uv_fs, int h,
                                                                 int w, int do_median, double* ou, double* ov,
                                                                 long long o_fs, long long o_rs, long long o_cs)
{
    __shared__ double sd[2][kXMedRows + 4][kXMedTx + 4];
    __shared__ float sk[2][kXMedRows + 4][kXMedTx + 4];
    const int f = blockIdx.z;
    const int x0 = blockIdx.x * kXMedTx, y0 = blockIdx.y * kXMedRows;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * kXMedTx + tx;
    const double* duf = du + (long long)f * s_fs;
    const double* dvf = dv + (long long)f * s_fs;
    if (do_median) {
        for (int i = tid; i < (kXMedRows + 4) * (kXMedTx + 4); i += kXMedTx * kXMedTy) {
            const int r = i / (kXMedTx + 4), c = i - r * (kXMedTx + 4);
            const int yy = mirror_x(min(y0 - 2 + r, h + 1), h);
            const int xx = mirror_x(min(x0 - 2 + c, w + 1), w);
            const long long o = (long long)yy * s_rs + xx;
            const double a = duf[o], b = dvf[o];
            sd[0][r][c] = a;
            sd[1][r][c] = b;
            sk[0][r][c] = hikey(a);
            sk[1][r][c] = hikey(b);
        }
        __syncthreads();
    }
    const int x = x0 + tx, ya = y0 + 2 * ty;
    if (x >= w || ya >= h) return;
    double m[2][2];  // [pixel a / b][du / dv]
    if (do_median) {
#pragma unroll
        for (int pl = 0; pl < 2; ++pl) {
            float c20[20], ea[5], eb[5];
#pragma unroll
            for (int dy = 0; dy < 4; ++dy)
#pragma unroll
                for (int dx = 0; dx < 5; ++dx) c20[dy * 5 + dx] = sk[pl][2 * ty + 1 + dy][tx + dx];
#pragma unroll
            for (int dx = 0; dx < 5; ++dx) {
                ea[dx] = sk[pl][2 * ty][tx + dx];
                eb[dx] = sk[pl][2 * ty + 5][tx + dx];
            }
            float km[2];
            median25_pair(c20, ea, eb, km[0], km[1]);
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int r0 = 2 * ty + q;
                int eq = 0, nlt = 0;
                bool finite = true;
                double pick = 0.0;
#pragma unroll
                for (int dy = 0; dy < 5; ++dy)
#pragma unroll
                    for (int dx = 0; dx < 5; ++dx) {
                        const float k = sk[pl][r0 + dy][tx + dx];
                        finite = finite && fabsf(k) <= 3.402823466e38f;
                        nlt += k < km[q];
                        if (k == km[q]) {
                            ++eq;
                            pick = sd[pl][r0 + dy][tx + dx];
                        }
                    }
                if (!(finite && eq == 1)) {
                    if (finite && km[q] != 0.0f) {
                        pick = median25_tie([&](int i) { return sd[pl][r0 + i / 5][tx + i % 5]; }, km[q], nlt, eq);
                    } else {
                        double win[25];
#pragma unroll
                        for (int dy = 0; dy < 5; ++dy)
#pragma unroll
                            for (int dx = 0; dx < 5; ++dx) win[dy * 5 + dx] = sd[pl][r0 + dy][tx + dx];
                        pick = median25d(win);
                    }
                }
                m[q][pl] = pick;
            }
        }
    } else {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int y = ya + q < h ? ya + q : ya;
            const long long o = (long long)y * s_rs + x;
            m[q][0] = duf[o];
            m[q][1] = dvf[o];
        }
    }
    const long long n = w + 2;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int y = ya + q;
        if (y >= h) break;
        const long long oc = (long long)(y + 1) * n + x + 1;
        ou[f * o_fs + y * o_rs + x * o_cs] = u ? dadd(u[f * uv_fs + oc], m[q][0]) : m[q][0];
        ov[f * o_fs + y * o_rs + x * o_cs] = v ? dadd(v[f * uv_fs + oc], m[q][1]) : m[q][1];
    }
}

cudaError_t launch_x_median5_plane(const double* src, int h, int w, double* dst, cudaStream_t st)
{
    dim3 blk(kXMedTx, kXMedTy), grd((w + kXMedTx - 1) / kXMedTx, (h + kXMedRows - 1) / kXMedRows, 1);
    const long long hw = (long long)h * w;
    kx_median_rm<<<grd, blk, 0, st>>>(src, src, hw, w, nullptr, nullptr, 0, h, w, 1, dst, dst, hw, w, 1);
    return cudaGetLastError();
}

cudaError_t launch_x_median_accum(const double* du, const double* dv, const double* u, const double* v,
                                  long long uv_fs, int n_frames, int h, int w, int do_median, double* ou, double* ov,
                                  long long o_fs, long long o_rs, long long o_cs, cudaStream_t st)
{
    if (n_frames > 65535) return cudaErrorInvalidValue;
    dim3 blk(kXMedTx, kXMedTy), grd((w + kXMedTx - 1) / kXMedTx, (h + kXMedRows - 1) / kXMedRows, n_frames);
    const long long n = w + 2, mn = (long long)(h + 2) * n;
    kx_median_rm<<<grd, blk, 0, st>>>(du + n + 1, dv + n + 1, mn, n, u, v, uv_fs, h, w, do_median, ou, ov, o_fs, o_rs,
                                      o_cs);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// GNC warping step update (core/optical_flow.py:745-755): u = u + du over the
// padded grid, then, when min(h, w) > 5, u = add_boundary(median5(u interior)).
// kx_gnc_median writes the new interior (strides o_fs, o_rs, o_cs) from the
// padded u, du; kx_gnc_ring then rewrites the padded u from it: the interior,
// and the border as the edge copy (median) or as u + du (no median).
// ---------------------------------------------------------------------------
__global__ void kx_gnc_median(const double* __restrict__ du, const double* __restrict__ dv,
                              const double* __restrict__ u, const double* __restrict__ v, long long uv_fs, int h, int w,
                              int do_median, double* ou, double* ov, long long o_fs, long long o_rs, long long o_cs)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int f = blockIdx.z;
    if (x >= w) return;
    const long long n = w + 2, mn = (long long)(h + 2) * n;
    const double* duf = du + (long long)f * mn;
    const double* dvf = dv + (long long)f * mn;
    const double* uf = u + f * uv_fs;
    const double* vf = v + f * uv_fs;
    double mu, mv;
    if (do_median) {
        double a[25], b[25];
        int q = 0;
        for (int dy = -2; dy <= 2; ++dy) {
            int yy = y + dy;
            if (yy < 0) yy = -yy;
            if (yy >= h) yy = 2 * (h - 1) - yy;
            for (int dx = -2; dx <= 2; ++dx) {
                int xx = x + dx;
                if (xx < 0) xx = -xx;
                if (xx >= w) xx = 2 * (w - 1) - xx;
                const long long o = (long long)(yy + 1) * n + xx + 1;
                a[q] = dadd(uf[o], duf[o]);
                b[q] = dadd(vf[o], dvf[o]);
                ++q;
            }
        }
        mu = median25_keys(a);
        mv = median25_keys(b);
    } else {
        const long long o = (long long)(y + 1) * n + x + 1;
        mu = dadd(uf[o], duf[o]);
        mv = dadd(vf[o], dvf[o]);
    }
    ou[f * o_fs + y * o_rs + x * o_cs] = mu;
    ov[f * o_fs + y * o_rs + x * o_cs] = mv;
}

__global__ void kx_gnc_ring(const double* __restrict__ au, const double* __restrict__ av, long long a_fs,
                            long long a_rs, long long a_cs, const double* __restrict__ du,
                            const double* __restrict__ dv, double* u, double* v, long long uv_fs, int h, int w,
                            int do_median)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // padded column
    const int j = blockIdx.y;                              // padded row
    const int f = blockIdx.z;
    const int n = w + 2;
    if (i >= n) return;
    const long long mn = (long long)(h + 2) * n, q = (long long)j * n + i;
    const bool interior = j >= 1 && j <= h && i >= 1 && i <= w;
    double* uf = u + f * uv_fs;
    double* vf = v + f * uv_fs;
    if (interior || do_median) {
        const long long a = f * a_fs + (long long)(xclamp(j, 1, h) - 1) * a_rs + (long long)(xclamp(i, 1, w) - 1) * a_cs;
        uf[q] = au[a];
        vf[q] = av[a];
    } else {
        uf[q] = dadd(uf[q], du[(long long)f * mn + q]);
        vf[q] = dadd(vf[q], dv[(long long)f * mn + q]);
    }
}

cudaError_t launch_x_gnc_update(const double* du, const double* dv, double* u, double* v, long long uv_fs,
                                int n_frames, int h, int w, int do_median, double* ou, double* ov, long long o_fs,
                                long long o_rs, long long o_cs, int write_ring, cudaStream_t st)
{
    dim3 blk(128), grd((w + 127) / 128, h, n_frames);
    kx_gnc_median<<<grd, blk, 0, st>>>(du, dv, u, v, uv_fs, h, w, do_median, ou, ov, o_fs, o_rs, o_cs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !write_ring) return e;
    dim3 grd2((w + 2 + 127) / 128, h + 2, n_frames);
    kx_gnc_ring<<<grd2, blk, 0, st>>>(ou, ov, o_fs, o_rs, o_cs, du, dv, u, v, uv_fs, h, w, do_median);
    return cudaGetLastError();
}

}  // namespace frg

namespace frg {

// ---------------------------------------------------------------------------
// Final upsampling of the flow when min_level > 0 (core/optical_flow.py:615-616,
// cv2.resize INTER_CUBIC): along one axis, output d samples the input at
// (d + 0.5) * in/out - 0.5 with four Keys (A = -0.75) float32 weights on
// clamped taps (tables built on the host).  Width pass first, then height,
// accumulating in the element type (float64 in parity mode).
// src planes (n, ih, iw) contiguous; the width pass writes (n, ih, ow)
// contiguous, the height pass writes through a strided view.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T addx(T a, T b);
template <>
__device__ __forceinline__ float addx<float>(float a, float b) { return a + b; }
template <>
__device__ __forceinline__ double addx<double>(double a, double b) { return __dadd_rn(a, b); }
template <typename T>
__device__ __forceinline__ T mulx(T a, T b);
template <>
__device__ __forceinline__ float mulx<float>(float a, float b) { return a * b; }
template <>
__device__ __forceinline__ double mulx<double>(double a, double b) { return __dmul_rn(a, b); }

template <typename T>
__global__ void k_cubic_up_w(const T* __restrict__ src, int n, int ih, int iw, T* __restrict__ dst, int ow,
                             const int32_t* __restrict__ s0, const float* __restrict__ wt)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, pl = blockIdx.z;
    if (x >= ow) return;
    const T* row = src + ((long long)pl * ih + y) * iw;
    T acc = (T)0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = xclamp(s0[x] - 1 + k, 0, iw - 1);
        acc = addx<T>(acc, mulx<T>(row[j], (T)wt[x * 4 + k]));
    }
    dst[((long long)pl * ih + y) * ow + x] = acc;
}

template <typename T>
__global__ void k_cubic_up_h(const T* __restrict__ src, int n_planes, int ih, int ow, T* __restrict__ dst,
                             long long fs, long long ps, long long rs, long long cs, int oh,
                             const int32_t* __restrict__ s0, const float* __restrict__ wt)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, fp = blockIdx.z;
    if (x >= ow) return;
    const T* col = src + (long long)fp * ih * ow + x;
    T acc = (T)0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = xclamp(s0[y] - 1 + k, 0, ih - 1);
        acc = addx<T>(acc, mulx<T>(col[(long long)j * ow], (T)wt[y * 4 + k]));
    }
    const int f = fp / n_planes, pl = fp - f * n_planes;
    dst[f * fs + pl * ps + (long long)y * rs + (long long)x * cs] = acc;
}

template <typename T>
cudaError_t launch_cubic_up(const T* src, int n_frames, int n_planes, int ih, int iw, T* tmp, T* dst, long long fs,
                            long long ps, long long rs, long long cs, int oh, int ow, const int32_t* sx,
                            const float* wx, const int32_t* sy, const float* wy, cudaStream_t st)
{
    dim3 blk(128);
    dim3 g1((ow + 127) / 128, ih, n_frames * n_planes);
    k_cubic_up_w<T><<<g1, blk, 0, st>>>(src, n_frames * n_planes, ih, iw, tmp, ow, sx, wx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 g2((ow + 127) / 128, oh, n_frames * n_planes);
    k_cubic_up_h<T><<<g2, blk, 0, st>>>(tmp, n_planes, ih, ow, dst, fs, ps, rs, cs, oh, sy, wy);
    return cudaGetLastError();
}

template cudaError_t launch_cubic_up<float>(const float*, int, int, int, int, float*, float*, long long, long long,
                                           long long, long long, int, int, const int32_t*, const float*,
                                           const int32_t*, const float*, cudaStream_t);
template cudaError_t launch_cubic_up<double>(const double*, int, int, int, int, double*, double*, long long,
                                            long long, long long, long long, int, int, const int32_t*, const float*,
                                            const int32_t*, const float*, cudaStream_t);

}  // namespace frg
