// CUDA kernels of the GB300 optical-flow path (sm_103a, FP32, no tensor cores).
//
// Every kernel follows one step of pyflowreg's get_displacement
// (src/pyflowreg/core/optical_flow.py:476-617); the reference line each one
// restates is given above it.  All kernels are bounded loops without
// inter-CTA waits, so none of them can hang.
#include "frg_internal.h"
#include "frg_select.cuh"

#include <math.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

namespace frg {

cudaError_t ensure_max_dyn_smem(const void* kernel, int bytes)
{
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> done;  // (kernel, device) -> bytes set
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(kernel, dev);
    const auto it = done.find(key);
    if (it != done.end() && it->second >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done[key] = bytes;
    return e;
}

cudaError_t ensure_nonportable_clusters(const void* kernel)
{
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, bool> done;  // (kernel, device)
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(kernel, dev);
    if (done.count(key)) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) done[key] = true;
    return e;
}

__constant__ float c_cubic[32 * 4];
__constant__ float c_linear[32 * 2];

cudaError_t upload_cubic_table(const float* tab128, const float* lin64)
{
    cudaError_t e = cudaMemcpyToSymbol(c_cubic, tab128, sizeof(float) * 128);
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_linear, lin64, sizeof(float) * 64);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ---------------------------------------------------------------------------
// Separable fused Gauss-cubic resize (util/resize_util.py:116-141, 232-254).
// Horizontal pass: dst[(f*n_planes + plane), y, x] = sum_p src[y, ix[x,p]] * wx[x,p]
// ---------------------------------------------------------------------------
__global__ void k_resize_h(View src, int n_planes, int ih, int iw, float* __restrict__ dst, int ow,
                           const int32_t* __restrict__ ix, const float* __restrict__ wx, int P)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int fp = blockIdx.z;
    if (x >= ow) return;
    const int f = fp / n_planes, pl = fp - f * n_planes;
    const float* row = src.p + f * src.fs + pl * src.ps + (long long)y * src.rs;
    const int32_t* ixr = ix + (long long)x * P;
    const float* wxr = wx + (long long)x * P;
    float s = 0.0f;
    for (int p = 0; p < P; ++p) s = fmaf(__ldg(row + (long long)ixr[p] * src.cs), wxr[p], s);
    dst[((long long)fp * ih + y) * ow + x] = s;
    (void)iw;
}


// Horizontal pass, row-block form: one block takes up to R input rows of one
// frame (all planes) into shared memory with asynchronous 16-byte copies
// (cp.async; the rows of an interleaved frame, or of each plane of a planar
// one, are one contiguous run), so every thread has its whole share of the
// block's bytes in flight at once.  Each thread then produces one (plane,
// output column) for RT consecutive rows, reading the tap table through L1;
// RT shrinks at the coarse levels (few output columns, many taps) so that
// every thread has work.  The sum is the same fmaf chain over the taps in
// order as k_resize_h, so the results are the same bits.
// mode 0: element-wise staging (any strides); 1: one contiguous interleaved
// run (cs == planes, rs == planes * iw); 2: one contiguous run per plane
// (cs == 1, rs == iw).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int RT>
__global__ void __launch_bounds__(256) k_resize_h_rows(View src, int n_planes, int ih, int iw, float* __restrict__ dst,
                                                       int ow, const int32_t* __restrict__ ix,
                                                       const float* __restrict__ wx, int P, int R, int mode)
{
    extern __shared__ __align__(16) float srow[];
    const int f = blockIdx.y;
    const int y0 = blockIdx.x * R;
    const int nr = min(R, ih - y0);
    const int tid = threadIdx.x, nth = blockDim.x;
    const int row_elems = n_planes * iw;
    const float* base = src.p + f * src.fs + (long long)y0 * src.rs;
    // shared layout: element (r, plane, x) at r * sr + plane * sp + x * sx
    const int sr = mode == 2 ? iw : row_elems, sp = mode == 2 ? nr * iw : 1, sx = mode == 2 ? 1 : n_planes;
    if (mode == 1) {
        const int n4 = (nr * row_elems) >> 2;
        for (int i = tid; i < n4; i += nth) cp_async16(srow + 4 * i, base + 4LL * i);
        cp_async_wait_all();
    } else if (mode == 2) {
        const int n4 = (nr * iw) >> 2;
        for (int pl = 0; pl < n_planes; ++pl) {
            const float* pb = base + pl * src.ps;
            for (int i = tid; i < n4; i += nth) cp_async16(srow + pl * sp + 4 * i, pb + 4LL * i);
        }
        cp_async_wait_all();
    } else {
        for (int i = tid; i < nr * row_elems; i += nth) {
            const int r = i / row_elems, rem = i - r * row_elems;
            const int x = rem / n_planes, pl = rem - x * n_planes;
            srow[r * sr + pl * sp + x * sx] = base[pl * src.ps + (long long)r * src.rs + (long long)x * src.cs];
        }
    }
    __syncthreads();
    const int groups = (nr + RT - 1) / RT;
    const int items = groups * n_planes * ow;
    for (int it = tid; it < items; it += nth) {
        const int x = it % ow, rest = it / ow;
        const int pl = rest % n_planes, r0 = (rest / n_planes) * RT;
        float acc[RT];
#pragma unroll
        for (int q = 0; q < RT; ++q) acc[q] = 0.0f;
        const int32_t* ixr = ix + (long long)x * P;
        const float* wxr = wx + (long long)x * P;
        const float* sb = srow + r0 * sr + pl * sp;
        for (int p = 0; p < P; ++p) {
            const float* sj = sb + __ldg(ixr + p) * sx;
            const float wgt = __ldg(wxr + p);
#pragma unroll
            for (int q = 0; q < RT; ++q)
                if (r0 + q < nr) acc[q] = fmaf(sj[q * sr], wgt, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < RT; ++q)
            if (r0 + q < nr) dst[(((long long)f * n_planes + pl) * ih + y0 + r0 + q) * ow + x] = acc[q];
    }
}

cudaError_t launch_resize_h(View src, int n_frames, int n_planes, int ih, int iw, float* dst, int ow,
                            const int32_t* ix, const float* wx, int P, cudaStream_t st)
{
    const long long row_bytes = (long long)n_planes * iw * 4;
    const int R = (int)std::min<long long>(std::min(16, ih), 49152 / row_bytes);
    if (R >= 1 && n_frames <= 65535) {
        const bool a16 = ((uintptr_t)src.p & 15) == 0 && (src.fs & 3) == 0;
        int mode = 0;
        if (a16 && src.cs == n_planes && src.ps == 1 && src.rs == (long long)n_planes * iw && (n_planes * iw) % 4 == 0)
            mode = 1;
        else if (a16 && src.cs == 1 && src.rs == iw && iw % 4 == 0 && (src.ps & 3) == 0)
            mode = 2;
        // rows per thread: the largest that still gives every thread of the block an output
        const int per_row = n_planes * ow;
        int RT = 8;
        while (RT > 1 && (long long)((R + RT - 1) / RT) * per_row < 256) RT >>= 1;
        const size_t smem = (size_t)R * row_bytes;
        dim3 grd((ih + R - 1) / R, n_frames);
        switch (RT) {
            case 8: k_resize_h_rows<8><<<grd, 256, smem, st>>>(src, n_planes, ih, iw, dst, ow, ix, wx, P, R, mode); break;
            case 4: k_resize_h_rows<4><<<grd, 256, smem, st>>>(src, n_planes, ih, iw, dst, ow, ix, wx, P, R, mode); break;
            case 2: k_resize_h_rows<2><<<grd, 256, smem, st>>>(src, n_planes, ih, iw, dst, ow, ix, wx, P, R, mode); break;
            default: k_resize_h_rows<1><<<grd, 256, smem, st>>>(src, n_planes, ih, iw, dst, ow, ix, wx, P, R, mode);
        }
        return cudaGetLastError();
    }
    dim3 blk(128), grd((ow + 127) / 128, ih, n_frames * n_planes);
    k_resize_h<<<grd, blk, 0, st>>>(src, n_planes, ih, iw, dst, ow, ix, wx, P);
    return cudaGetLastError();
}

// Vertical pass; with pad = 1 the output is the level array with a one-pixel
// edge-replicated ring (add_boundary, core/optical_flow.py:48-70).  Four
// output rows per thread: the four tap chains are independent, so each
// thread keeps four sets of column loads in flight (one output per thread is
// bound by the latency of its short chain).  The sum per output is the same
// fmaf chain over the taps in order.
constexpr int kRvRows = 4;

__global__ void k_resize_v4(const float* __restrict__ src, int n_planes, int ih, int ow, ViewW dst, int oh, int pad,
                            const int32_t* __restrict__ iy, const float* __restrict__ wy, int P)
{
    const int xo = blockIdx.x * blockDim.x + threadIdx.x;
    const int yo0 = blockIdx.y * kRvRows;
    const int fp = blockIdx.z;
    const int ohp = oh + 2 * pad;
    if (xo >= ow + 2 * pad) return;
    const int x = clampi(xo - pad, 0, ow - 1);
    const float* col = src + (long long)fp * ih * ow + x;
    const int32_t* iyr[kRvRows];
    const float* wyr[kRvRows];
#pragma unroll
    for (int q = 0; q < kRvRows; ++q) {
        const int y = clampi(min(yo0 + q, ohp - 1) - pad, 0, oh - 1);
        iyr[q] = iy + (long long)y * P;
        wyr[q] = wy + (long long)y * P;
    }
    float s[kRvRows];
#pragma unroll
    for (int q = 0; q < kRvRows; ++q) s[q] = 0.0f;
    for (int p = 0; p < P; ++p) {
#pragma unroll
        for (int q = 0; q < kRvRows; ++q) s[q] = fmaf(__ldg(col + (long long)iyr[q][p] * ow), wyr[q][p], s[q]);
    }
    const int f = fp / n_planes, pl = fp - f * n_planes;
#pragma unroll
    for (int q = 0; q < kRvRows; ++q)
        if (yo0 + q < ohp) dst.p[f * dst.fs + pl * dst.ps + (long long)(yo0 + q) * dst.rs + (long long)xo * dst.cs] = s[q];
}

cudaError_t launch_resize_v(const float* src, int n_frames, int n_planes, int ih, int ow, ViewW dst,
                            int oh, int pad, const int32_t* iy, const float* wy, int P, cudaStream_t st)
{
    const int owp = ow + 2 * pad, ohp = oh + 2 * pad;
    const int bx = owp >= 96 ? 128 : (owp >= 48 ? 64 : 32);
    dim3 blk(bx), grd((owp + bx - 1) / bx, (ohp + kRvRows - 1) / kRvRows, n_frames * n_planes);
    k_resize_v4<<<grd, blk, 0, st>>>(src, n_planes, ih, ow, dst, oh, pad, iy, wy, P);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Backward warp with out-of-bounds fill (core/warping.py:160-234): the map is
// x + u / h_col, y + v / h_row in float32; points outside [0, W) x [0, H)
// take the reference level value; the rest is clamped and sampled on the
// 1/32-pixel grid of cv2.remap (round half to even) with Keys A = -0.75
// bicubic or bilinear weights and replicated borders.
// ---------------------------------------------------------------------------
// The interpolation tables are read per lane at the lane's own sub-pixel
// position, so they are copied into shared memory first (constant memory
// serialises a warp's distinct addresses); the 4 x 4 weights of a pixel are
// formed once for all channels.
__global__ void k_warp(View f2, View f1, View u, View v, int K, int h, int w, float h_col, float h_row,
                       int cubic, ViewW out)
{
    __shared__ float s_tab[32 * 4];
    for (int i = threadIdx.x; i < 32 * 4; i += blockDim.x) s_tab[i] = cubic ? c_cubic[i] : (i < 64 ? c_linear[i] : 0.0f);
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int f = blockIdx.z;
    if (x >= w) return;
    const float uu = u.p[f * u.fs + (long long)y * u.rs + (long long)x * u.cs];
    const float vv = v.p[f * v.fs + (long long)y * v.rs + (long long)x * v.cs];
    const float mx = __fadd_rn((float)x, __fdiv_rn(uu, h_col));
    const float my = __fadd_rn((float)y, __fdiv_rn(vv, h_row));
    const bool oob = (mx < 0.0f) || (mx >= (float)w) || (my < 0.0f) || (my >= (float)h);
    if (oob) {
        for (int k = 0; k < K; ++k)
            out.p[f * out.fs + k * out.ps + (long long)y * out.rs + (long long)x * out.cs] =
                f1.p[f * f1.fs + k * f1.ps + (long long)y * f1.rs + (long long)x * f1.cs];
        return;
    }
    const float cx = fminf(fmaxf(mx, 0.0f), (float)(w - 1));
    const float cy = fminf(fmaxf(my, 0.0f), (float)(h - 1));
    const int X = __float2int_rn(cx * 32.0f);
    const int Y = __float2int_rn(cy * 32.0f);
    const int ix = X >> 5, fx = X & 31;
    const int iy = Y >> 5, fy = Y & 31;
    if (cubic) {
        float w2[4][4];
        long long ro[4], co[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float wyi = s_tab[fy * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) w2[i][j] = __fmul_rn(wyi, s_tab[fx * 4 + j]);
            ro[i] = (long long)clampi(iy - 1 + i, 0, h - 1) * f2.rs;
            co[i] = (long long)clampi(ix - 1 + i, 0, w - 1) * f2.cs;
        }
        for (int k = 0; k < K; ++k) {
            const float* src = f2.p + f * f2.fs + k * f2.ps;
            float acc = 0.0f;
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc = fmaf(src[ro[i] + co[j]], w2[i][j], acc);
            out.p[f * out.fs + k * out.ps + (long long)y * out.rs + (long long)x * out.cs] = acc;
        }
    } else {
        float w2[2][2];
        long long ro[2], co[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const float wyi = s_tab[fy * 2 + i];
#pragma unroll
            for (int j = 0; j < 2; ++j) w2[i][j] = __fmul_rn(wyi, s_tab[fx * 2 + j]);
            ro[i] = (long long)clampi(iy + i, 0, h - 1) * f2.rs;
            co[i] = (long long)clampi(ix + i, 0, w - 1) * f2.cs;
        }
        for (int k = 0; k < K; ++k) {
            const float* src = f2.p + f * f2.fs + k * f2.ps;
            float acc = 0.0f;
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) acc = fmaf(src[ro[i] + co[j]], w2[i][j], acc);
            out.p[f * out.fs + k * out.ps + (long long)y * out.rs + (long long)x * out.cs] = acc;
        }
    }
}

cudaError_t launch_warp(View f2, View f1, View u, View v, int n_frames, int K, int h, int w,
                        float h_col, float h_row, int cubic, ViewW out, cudaStream_t st)
{
    dim3 blk(128), grd((w + 127) / 128, h, n_frames);
    k_warp<<<grd, blk, 0, st>>>(f2, f1, u, v, K, h, w, h_col, h_row, cubic, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Motion tensor (core/optical_flow.py:73-160 gradient constancy, 163-228
// gray-value constancy).  Derivatives use the reference's one-pixel symmetric
// padding: every neighbour index is clamped into the level.  Output is
// diagonal-major, per frame [6][K][D*P] in the order J11, J22, J33, J12, J13, J23.
// ---------------------------------------------------------------------------
// J11..J23 of channel k at pixel (y, x) of frame f.
__device__ __forceinline__ void tensor_at(const View& f1, const View& f2, int f, int k, int y, int x, int h, int w,
                                          float hy, float hx, int gray, float* out)
{
    const int xm = max(x - 1, 0), xp = min(x + 1, w - 1);
    const int ym = max(y - 1, 0), yp = min(y + 1, h - 1);
    const float h2x = 2.0f * hx, h2y = 2.0f * hy;
    const float hxx = hx * hx, hyy = hy * hy;
    {
        const float* a = f1.p + f * f1.fs + k * f1.ps;
        const float* b = f2.p + f * f2.fs + k * f2.ps;
#define A_(r, c) a[(long long)(r) * f1.rs + (long long)(c) * f1.cs]
#define B_(r, c) b[(long long)(r) * f2.rs + (long long)(c) * f2.cs]
        float j11, j22, j33, j12, j13, j23;
        if (gray) {
            const float fxv = 0.5f * ((A_(y, xp) - A_(y, xm)) / h2x + (B_(y, xp) - B_(y, xm)) / h2x);
            const float fyv = 0.5f * ((A_(yp, x) - A_(ym, x)) / h2y + (B_(yp, x) - B_(ym, x)) / h2y);
            const float ftv = B_(y, x) - A_(y, x);
            j11 = fxv * fxv; j22 = fyv * fyv; j33 = ftv * ftv;
            j12 = fxv * fyv; j13 = fxv * ftv; j23 = fyv * ftv;
        } else {
            const float fx_m = 0.5f * ((A_(ym, xp) - A_(ym, xm)) / h2x + (B_(ym, xp) - B_(ym, xm)) / h2x);
            const float fx_p = 0.5f * ((A_(yp, xp) - A_(yp, xm)) / h2x + (B_(yp, xp) - B_(yp, xm)) / h2x);
            const float fxy = (fx_p - fx_m) / h2y;
            const float ft_l = B_(y, xm) - A_(y, xm), ft_r = B_(y, xp) - A_(y, xp);
            const float ft_u = B_(ym, x) - A_(ym, x), ft_d = B_(yp, x) - A_(yp, x);
            const float fxt = (ft_r - ft_l) / h2x;
            const float fyt = (ft_d - ft_u) / h2y;
            const float a0 = A_(y, x), b0 = B_(y, x);
            const float fxx = 0.5f * (((A_(y, xm) - a0) + (A_(y, xp) - a0)) / hxx +
                                      ((B_(y, xm) - b0) + (B_(y, xp) - b0)) / hxx);
            const float fyy = 0.5f * (((A_(ym, x) - a0) + (A_(yp, x) - a0)) / hyy +
                                      ((B_(ym, x) - b0) + (B_(yp, x) - b0)) / hyy);
            const float reg_x = 1.0f / (fxx * fxx + fxy * fxy + 1e-6f);
            const float reg_y = 1.0f / (fxy * fxy + fyy * fyy + 1e-6f);
            j11 = reg_x * fxx * fxx + reg_y * fxy * fxy;
            j22 = reg_x * fxy * fxy + reg_y * fyy * fyy;
            j33 = reg_x * fxt * fxt + reg_y * fyt * fyt;
            j12 = reg_x * fxx * fxy + reg_y * fxy * fyy;
            j13 = reg_x * fxx * fxt + reg_y * fxy * fyt;
            j23 = reg_x * fxy * fxt + reg_y * fyy * fyt;
        }
#undef A_
#undef B_
        out[0] = j11;
        out[1] = j22;
        out[2] = j33;
        out[3] = j12;
        out[4] = j13;
        out[5] = j23;
    }
}

__global__ void k_tensor(View f1, View f2, int K, int h, int w, float hy, float hx, int gray,
                         float* __restrict__ J, long long J_fs, DiagGeom g)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int f = blockIdx.z;
    if (x >= w) return;
    const long long di = diag_index(g, y, x);
    const long long plane = (long long)g.D * g.P;
    const long long qs = (long long)K * plane;
    float* Jf = J + f * J_fs;
    for (int k = 0; k < K; ++k) {
        float j[6];
        tensor_at(f1, f2, f, k, y, x, h, w, hy, hx, gray, j);
        const long long kb = (long long)k * plane + di;
#pragma unroll
        for (int q = 0; q < 6; ++q) Jf[q * qs + kb] = j[q];
    }
}

// Constant part of the smoothness numerator at level pixel (y, x) from the
// edge-padded (h+2) x (w+2) u, v (core/level_solver.py:317-340):
//   lap_u = wx*((uL-uc)+(uR-uc)) + wy*((uU-uc)+(uD-uc)), lap_v likewise.
__device__ __forceinline__ void lap_at(const View& u, const View& v, int f, int y, int x, float wx, float wy,
                                       float& lu, float& lv)
{
    const float* up = u.p + f * u.fs;
    const float* vp = v.p + f * v.fs;
#define U_(r, c) up[(long long)(r) * u.rs + (long long)(c) * u.cs]
#define V_(r, c) vp[(long long)(r) * v.rs + (long long)(c) * v.cs]
    const float uc = U_(y + 1, x + 1), vc = V_(y + 1, x + 1);
    lu = wx * ((U_(y + 1, x) - uc) + (U_(y + 1, x + 2) - uc)) + wy * ((U_(y, x + 1) - uc) + (U_(y + 2, x + 1) - uc));
    lv = wx * ((V_(y + 1, x) - vc) + (V_(y + 1, x + 2) - vc)) + wy * ((V_(y, x + 1) - vc) + (V_(y + 2, x + 1) - vc));
#undef U_
#undef V_
}

// Tiled form: a 32 x 32 pixel tile is computed into shared memory, then every
// diagonal crossing the tile is written as one contiguous run of the
// diagonal-major layout (up to 128 bytes per warp store instead of 32
// scattered 4-byte stores).  Row pitch 34: the row writes (lane = column) and
// the anti-diagonal reads (lane = row, column falling, word step 33) both hit
// 32 different banks.
constexpr int kTensTile = 32;
constexpr int kTensLd = kTensTile + 2;

__global__ void __launch_bounds__(256, 3) k_tensor_tiled(View f1, View f2, int K, int h, int w, float hy, float hx,
                                                      int gray, float* __restrict__ J, long long J_fs, DiagGeom g,
                                                      View u, View v, float wx, float wy, float* __restrict__ lap,
                                                      long long lap_fs)
{
    extern __shared__ float tile[];  // [6K (+2 with lap)][32][34]
    const int f = blockIdx.z;
    const int r0 = blockIdx.y * kTensTile, c0 = blockIdx.x * kTensTile;
    const int tx = threadIdx.x & 31, tw = threadIdx.x >> 5;  // 8 warps
    const int ld = kTensLd;
    const int nq = 6 * K + (lap ? 2 : 0);
    for (int rr = tw; rr < kTensTile; rr += 8) {
        const int y = r0 + rr, x = c0 + tx;
        if (y < h && x < w) {
            for (int k = 0; k < K; ++k) {
                float j[6];
                tensor_at(f1, f2, f, k, y, x, h, w, hy, hx, gray, j);
#pragma unroll
                for (int q = 0; q < 6; ++q) tile[((q * K + k) * kTensTile + rr) * ld + tx] = j[q];
            }
            if (lap) {
                float lu, lv;
                lap_at(u, v, f, y, x, wx, wy, lu, lv);
                tile[((6 * K) * kTensTile + rr) * ld + tx] = lu;
                tile[((6 * K + 1) * kTensTile + rr) * ld + tx] = lv;
            }
        }
    }
    __syncthreads();
    const long long plane = (long long)g.D * g.P;
    float* Jf = J + f * J_fs;
    float* Lf = lap ? lap + f * lap_fs : nullptr;
    // local diagonal dd = rr + cc in [0, 62]; rows of the segment are contiguous
    for (int dd = tw; dd < 2 * kTensTile - 1; dd += 8) {
        const int rr_lo = max(0, dd - (kTensTile - 1));
        const int rr = rr_lo + tx;
        const int cc = dd - rr;
        if (rr > min(kTensTile - 1, dd)) continue;
        const int y = r0 + rr, x = c0 + cc;
        if (y >= h || x >= w) continue;
        const long long di = diag_index(g, y, x);
        for (int qk = 0; qk < 6 * K; ++qk) Jf[(long long)qk * plane + di] = tile[(qk * kTensTile + rr) * ld + cc];
        for (int qk = 6 * K; qk < nq; ++qk)
            Lf[(long long)(qk - 6 * K) * plane + di] = tile[(qk * kTensTile + rr) * ld + cc];
    }
}

namespace {

cudaError_t run_tensor(View f1, View f2, int n_frames, int K, int h, int w, float hy, float hx, int gray, float* J,
                       long long J_fs, DiagGeom g, View u, View v, float wx, float wy, float* lap, long long lap_fs,
                       cudaStream_t st)
{
    const size_t smem = (size_t)(6 * K + (lap ? 2 : 0)) * kTensTile * kTensLd * sizeof(float);
    if (smem <= 200 * 1024) {
        {
            const cudaError_t e = ensure_max_dyn_smem((const void*)k_tensor_tiled, 200 * 1024);
            if (e != cudaSuccess) return e;
        }
        dim3 grd((w + kTensTile - 1) / kTensTile, (h + kTensTile - 1) / kTensTile, n_frames);
        k_tensor_tiled<<<grd, 256, smem, st>>>(f1, f2, K, h, w, hy, hx, gray, J, J_fs, g, u, v, wx, wy, lap, lap_fs);
        return cudaGetLastError();
    }
    dim3 blk(128), grd((w + 127) / 128, h, n_frames);
    k_tensor<<<grd, blk, 0, st>>>(f1, f2, K, h, w, hy, hx, gray, J, J_fs, g);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !lap) return e;
    return launch_lap(u, v, n_frames, h, w, wx, wy, lap, lap_fs, g, st);
}

}  // namespace

cudaError_t launch_tensor(View f1, View f2, int n_frames, int K, int h, int w, float hy, float hx,
                          int gray, float* J, long long J_fs, DiagGeom g, cudaStream_t st)
{
    return run_tensor(f1, f2, n_frames, K, h, w, hy, hx, gray, J, J_fs, g, View{}, View{}, 0.0f, 0.0f, nullptr, 0,
                      st);
}

cudaError_t launch_tensor_lap(View f1, View f2, int n_frames, int K, int h, int w, float hy, float hx, int gray,
                              float* J, long long J_fs, DiagGeom g, View u, View v, float wx, float wy, float* lap,
                              long long lap_fs, cudaStream_t st)
{
    return run_tensor(f1, f2, n_frames, K, h, w, hy, hx, gray, J, J_fs, g, u, v, wx, wy, lap, lap_fs, st);
}

// ---------------------------------------------------------------------------
// Constant part of the smoothness numerator for a level (u, v fixed during
// the solve; core/level_solver.py:317-340):
//   lap_u = wx*((uL-uc)+(uR-uc)) + wy*((uU-uc)+(uD-uc)), lap_v likewise,
// from the edge-padded (h+2) x (w+2) u, v; diagonal-major output [2][D*P].
// ---------------------------------------------------------------------------
__global__ void k_lap(View u, View v, int h, int w, float wx, float wy, float* __restrict__ lap,
                      long long lap_fs, DiagGeom g)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int f = blockIdx.z;
    if (x >= w) return;
    float lu, lv;
    lap_at(u, v, f, y, x, wx, wy, lu, lv);
    const long long di = diag_index(g, y, x);
    const long long plane = (long long)g.D * g.P;
    lap[f * lap_fs + di] = lu;
    lap[f * lap_fs + plane + di] = lv;
    (void)h;
}

cudaError_t launch_lap(View u, View v, int n_frames, int h, int w, float wx, float wy, float* lap,
                       long long lap_fs, DiagGeom g, cudaStream_t st)
{
    dim3 blk(128), grd((w + 127) / 128, h, n_frames);
    k_lap<<<grd, blk, 0, st>>>(u, v, h, w, wx, wy, lap, lap_fs, g);
    return cudaGetLastError();
}

// Row-major planes -> diagonal-major planes: dst[f][plane][D*P].
__global__ void k_to_diag(View src, int n_planes, int h, int w, float* __restrict__ dst,
                          long long dst_fs, DiagGeom g)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int fp = blockIdx.z;
    if (x >= w) return;
    const int f = fp / n_planes, pl = fp - f * n_planes;
    const float val = src.p[f * src.fs + pl * src.ps + (long long)y * src.rs + (long long)x * src.cs];
    dst[f * dst_fs + (long long)pl * g.D * g.P + diag_index(g, y, x)] = val;
    (void)h;
}

cudaError_t launch_to_diag(View src, int n_frames, int n_planes, int h, int w, float* dst,
                           long long dst_fs, DiagGeom g, cudaStream_t st)
{
    dim3 blk(128), grd((w + 127) / 128, h, n_frames * n_planes);
    k_to_diag<<<grd, blk, 0, st>>>(src, n_planes, h, w, dst, dst_fs, g);
    return cudaGetLastError();
}

// Diagonal-major planes -> row-major planes with a `ring`-pixel border:
// ring_mode 0 leaves the border untouched, 1 zeroes it, 2 copies the nearest
// interior value (the Neumann copy of set_boundary_2d).
__global__ void k_from_diag(const float* __restrict__ src, long long src_fs, int n_planes, DiagGeom g,
                            ViewW dst, int ring, int ring_mode)
{
    const int xo = blockIdx.x * blockDim.x + threadIdx.x;
    const int yo = blockIdx.y;
    const int fp = blockIdx.z;
    const int W2 = g.w + 2 * ring, H2 = g.h + 2 * ring;
    if (xo >= W2) return;
    const int f = fp / n_planes, pl = fp - f * n_planes;
    const int x = xo - ring, y = yo - ring;
    const bool inside = x >= 0 && x < g.w && y >= 0 && y < g.h;
    if (!inside && ring_mode == 0) return;
    float val = 0.0f;
    if (inside || ring_mode == 2) {
        const int xc = clampi(x, 0, g.w - 1), yc = clampi(y, 0, g.h - 1);
        val = src[f * src_fs + (long long)pl * g.D * g.P + diag_index(g, yc, xc)];
    }
    dst.p[f * dst.fs + pl * dst.ps + (long long)yo * dst.rs + (long long)xo * dst.cs] = val;
    (void)H2;
}

cudaError_t launch_from_diag(const float* src, long long src_fs, int n_frames, int n_planes, DiagGeom g,
                             ViewW dst, int ring, int ring_mode, cudaStream_t st)
{
    dim3 blk(128), grd((g.w + 2 * ring + 127) / 128, g.h + 2 * ring, n_frames * n_planes);
    k_from_diag<<<grd, blk, 0, st>>>(src, src_fs, n_planes, g, dst, ring, ring_mode);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Coefficient fold at a lagged-nonlinearity tick (core/level_solver.py:229-255,
// 342-364).  mode bit 0: first pass, du = dv = 0; bit 1: psi from the current
// (du, dv) (a tick), else psi = 1.  Writes, per pixel, the five coefficients the SOR update
// needs: A12 = sum_k W psi J12, BU = lap_u - sum_k W psi J13,
// BV = lap_v - sum_k W psi J23, 1/den_u, 1/den_v (0 where the denominator is 0).
// ---------------------------------------------------------------------------
struct AData { float a[kMaxK]; };

__global__ void k_fold(const float* __restrict__ J, long long J_fs, const float* __restrict__ W,
                       long long W_fs, const float* __restrict__ lap, long long lap_fs,
                       float* __restrict__ du, float* __restrict__ dv, long long st_fs,
                       float* __restrict__ coef, long long coef_fs, int K, DiagGeom g, AData ad,
                       int mode, float wx, float wy)
{
    const long long plane = (long long)g.D * g.P;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (i >= plane) return;
    const int d = (int)(i / g.P);
    const int r = (int)(i - (long long)d * g.P);
    const int c = d - r;
    if (r >= g.h || c < 0 || c >= g.w) return;
    float* duf = du + f * st_fs;
    float* dvf = dv + f * st_fs;
    const bool zero_init = (mode & 1) != 0;
    const bool tick = (mode & 2) != 0;
    float a = 0.0f, b = 0.0f;
    if (zero_init) {
        duf[i] = 0.0f;
        dvf[i] = 0.0f;
    } else {
        a = duf[i];
        b = dvf[i];
    }
    const float* Jf = J + f * J_fs;
    const float* Wf = W + f * W_fs;
    const long long qs = (long long)K * plane;
    float A11 = 0.f, A22 = 0.f, A12 = 0.f, C13 = 0.f, C23 = 0.f;
    for (int k = 0; k < K; ++k) {
        const long long o = (long long)k * plane + i;
        const float j11 = Jf[o], j22 = Jf[qs + o], j33 = Jf[2 * qs + o];
        const float j12 = Jf[3 * qs + o], j13 = Jf[4 * qs + o], j23 = Jf[5 * qs + o];
        float psi = 1.0f;
        if (tick) {
            float E = j11 * a * a + j22 * b * b + j23 * b + 2.0f * j12 * a * b + 2.0f * j13 * a + j23 * b + j33;
            E = fmaxf(E, 0.0f);
            psi = ad.a[k] * powf(E + 1e-5f, ad.a[k] - 1.0f);
        }
        const float wp = Wf[o] * psi;
        A11 = fmaf(wp, j11, A11);
        A22 = fmaf(wp, j22, A22);
        A12 = fmaf(wp, j12, A12);
        C13 = fmaf(wp, j13, C13);
        C23 = fmaf(wp, j23, C23);
    }
    const float sm = ((wx + wx) + wy) + wy;
    const float den_u = sm + A11, den_v = sm + A22;
    float* cf = coef + f * coef_fs;
    cf[i] = A12;
    cf[plane + i] = lap[f * lap_fs + i] - C13;
    cf[2 * plane + i] = lap[f * lap_fs + plane + i] - C23;
    cf[3 * plane + i] = den_u != 0.0f ? 1.0f / den_u : 0.0f;
    cf[4 * plane + i] = den_v != 0.0f ? 1.0f / den_v : 0.0f;
}

cudaError_t launch_fold(const float* J, long long J_fs, const float* W, long long W_fs,
                        const float* lap, long long lap_fs, float* du, float* dv,
                        long long st_fs, float* coef, long long coef_fs, int n_frames, int K,
                        DiagGeom g, const float* a_data, int mode, float wx, float wy,
                        cudaStream_t st)
{
    AData ad;
    for (int k = 0; k < kMaxK; ++k) ad.a[k] = k < K ? a_data[k] : 0.0f;
    const long long plane = (long long)g.D * g.P;
    dim3 blk(256), grd((unsigned)((plane + 255) / 256), n_frames);
    k_fold<<<grd, blk, 0, st>>>(J, J_fs, W, W_fs, lap, lap_fs, du, dv, st_fs, coef, coef_fs, K, g, ad,
                                mode, wx, wy);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Exact-order SOR (core/level_solver.py:257-364) as a pipelined wavefront.
//
// The reference sweeps columns outer, rows inner, in place, so the update of
// pixel (r, c) in iteration t reads iteration t values at (r-1, c), (r, c-1)
// and iteration t-1 values at (r+1, c), (r, c+1).  Processing (r, c, t) at
// step s = r + c + 2t satisfies all four dependencies with a one-step gap, and
// at any step the pixels being written (diagonals of s's parity) and the
// pixels being read (the other parity) are disjoint.  Neighbours across the
// level border read the pixel's own pre-update value (the Neumann copy of
// set_boundary_2d, :45-66, taken at the start of the iteration).
//
// One CTA owns one frame of the level for G consecutive iterations (the span
// between two psi ticks).  Thread a owns row a.  A shared-memory ring keeps the
// 2G+2 diagonals that are live; diagonal s+2 is stored into the ring at step s
// from registers filled kPrefetch steps earlier, and the diagonal that leaves
// the ring is written back to global memory.
// Ring slot layout: 7 planes of P floats: du, dv, A12, BU, BV, 1/den_u, 1/den_v.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kMaxLane) k_sor(const float* __restrict__ coef, long long coef_fs,
                                                  float* __restrict__ du_g, float* __restrict__ dv_g,
                                                  long long st_fs, DiagGeom g, int G, float wa, float wb,
                                                  float omega)
{
    extern __shared__ float sm[];
    const int P = g.P, A = g.h, B = g.w, D = g.D;
    const int R = 2 * G + 2;
    const int a = threadIdx.x;
    const long long plane = (long long)D * P;
    const float* cf = coef + blockIdx.x * coef_fs;
    float* du = du_g + blockIdx.x * st_fs;
    float* dv = dv_g + blockIdx.x * st_fs;
    const float one_m_omega = 1.0f - omega;

    auto row_valid = [&](int d) { return d >= 0 && d < D && a < A && a <= d && d - a < B; };
    auto load = [&](int d, float* r) {
        if (row_valid(d)) {
            const long long o = (long long)d * P + a;
            r[0] = du[o];
            r[1] = dv[o];
#pragma unroll
            for (int q = 0; q < 5; ++q) r[2 + q] = cf[q * plane + o];
        }
    };
    auto put = [&](int d, const float* r) {
        if (row_valid(d)) {
            float* S = sm + (long long)(d % R) * 7 * P + a;
#pragma unroll
            for (int q = 0; q < 7; ++q) S[q * P] = r[q];
        }
    };
    auto writeback = [&](int d) {
        if (row_valid(d)) {
            const float* S = sm + (long long)(d % R) * 7 * P + a;
            const long long o = (long long)d * P + a;
            du[o] = S[0];
            dv[o] = S[P];
        }
    };

    float buf[kPrefetch][7];
    {
        float r0[7], r1[7];
        load(0, r0);
        load(1, r1);
        put(0, r0);
        put(1, r1);
    }
#pragma unroll
    for (int j = 0; j < kPrefetch; ++j) load(2 + j, buf[(2 + j) % kPrefetch]);
    __syncthreads();

    const int nsteps = D + 2 * (G - 1);
    for (int s0 = 0; s0 < nsteps; s0 += kPrefetch) {
#pragma unroll
        for (int q = 0; q < kPrefetch; ++q) {
            const int s = s0 + q;
            if (s < nsteps) {
                for (int gi = 0; gi < G; ++gi) {
                    const int d = s - 2 * gi;
                    if (d < 0) break;
                    if (d >= D) continue;
                    const int b = d - a;
                    if (a >= A || b < 0 || b >= B) continue;
                    float* S = sm + (long long)(d % R) * 7 * P;
                    const float* Sm = sm + (long long)((d + R - 1) % R) * 7 * P;
                    const float* Sp = sm + (long long)((d + 1) % R) * 7 * P;
                    const float duc = S[a], dvc = S[P + a];
                    const float A12 = S[2 * P + a], BU = S[3 * P + a], BV = S[4 * P + a];
                    const float iDu = S[5 * P + a], iDv = S[6 * P + a];
                    const float duAm = a > 0 ? Sm[a - 1] : duc;
                    const float dvAm = a > 0 ? Sm[P + a - 1] : dvc;
                    const float duBm = b > 0 ? Sm[a] : duc;
                    const float dvBm = b > 0 ? Sm[P + a] : dvc;
                    const float duAp = a < A - 1 ? Sp[a + 1] : duc;
                    const float dvAp = a < A - 1 ? Sp[P + a + 1] : dvc;
                    const float duBp = b < B - 1 ? Sp[a] : duc;
                    const float dvBp = b < B - 1 ? Sp[P + a] : dvc;
                    const float nu = wa * (duAm + duAp) + wb * (duBm + duBp) + BU - A12 * dvc;
                    const float dun = one_m_omega * duc + omega * (nu * iDu);
                    const float nv = wa * (dvAm + dvAp) + wb * (dvBm + dvBp) + BV - A12 * dun;
                    const float dvn = one_m_omega * dvc + omega * (nv * iDv);
                    S[a] = dun;
                    S[P + a] = dvn;
                }
                writeback(s - 2 * G);
                put(s + 2, buf[(q + 2) % kPrefetch]);
                load(s + 2 + kPrefetch, buf[(q + 2) % kPrefetch]);
            }
            __syncthreads();
        }
    }
    for (int e = max(0, nsteps - 2 * G); e < D; ++e) writeback(e);
}

cudaError_t launch_sor(const float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                       int n_frames, DiagGeom g, int G, float wa, float wb, float omega,
                       cudaStream_t st)
{
    if (g.P > kMaxLane || G < 1 || G > kGMax || (g.P & 31)) return cudaErrorInvalidValue;
    const int R = 2 * G + 2;
    const size_t smem = (size_t)R * 7 * g.P * sizeof(float);
    {
        const cudaError_t e =
            ensure_max_dyn_smem((const void*)k_sor, (int)((size_t)kRing * 7 * kMaxLane * sizeof(float)));
        if (e != cudaSuccess) return e;
    }
    k_sor<<<n_frames, g.P, smem, st>>>(coef, coef_fs, du, dv, st_fs, g, G, wa, wb, omega);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The same pass for levels too tall for a shared-memory ring: du, dv and the
// folded coefficients stay in global memory (diagonal-major); one CTA per
// frame walks the wavefront, each step's pixels spread over its threads.
// __syncthreads orders one step's stores before the next step's loads.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_sor_global(const float* __restrict__ coef, long long coef_fs,
                                                      float* du_g, float* dv_g, long long st_fs, DiagGeom g, int G,
                                                      float wa, float wb, float omega)
{
    const int P = g.P, A = g.h, B = g.w, D = g.D;
    const long long plane = (long long)D * P;
    const float* cf = coef + blockIdx.x * coef_fs;
    float* du = du_g + blockIdx.x * st_fs;
    float* dv = dv_g + blockIdx.x * st_fs;
    const float one_m_omega = 1.0f - omega;
    const int nsteps = D + 2 * (G - 1);
    for (int s = 0; s < nsteps; ++s) {
        for (int gi = 0; gi < G; ++gi) {
            const int d = s - 2 * gi;
            if (d < 0) break;
            if (d >= D) continue;
            const int r0 = d - (B - 1) > 0 ? d - (B - 1) : 0;
            const int r1 = d < A - 1 ? d : A - 1;
            for (int a = r0 + threadIdx.x; a <= r1; a += blockDim.x) {
                const int b = d - a;
                const long long o = (long long)d * P + a;
                const long long om = o - P, op = o + P;  // same row on diagonals d - 1, d + 1
                const float duc = du[o], dvc = dv[o];
                const float duAm = a > 0 ? du[om - 1] : duc, dvAm = a > 0 ? dv[om - 1] : dvc;
                const float duBm = b > 0 ? du[om] : duc, dvBm = b > 0 ? dv[om] : dvc;
                const float duAp = a < A - 1 ? du[op + 1] : duc, dvAp = a < A - 1 ? dv[op + 1] : dvc;
                const float duBp = b < B - 1 ? du[op] : duc, dvBp = b < B - 1 ? dv[op] : dvc;
                const float A12 = cf[o], BU = cf[plane + o], BV = cf[2 * plane + o];
                const float iDu = cf[3 * plane + o], iDv = cf[4 * plane + o];
                const float nu = wa * (duAm + duAp) + wb * (duBm + duBp) + BU - A12 * dvc;
                const float dun = one_m_omega * duc + omega * (nu * iDu);
                const float nv = wa * (dvAm + dvAp) + wb * (dvBm + dvBp) + BV - A12 * dun;
                const float dvn = one_m_omega * dvc + omega * (nv * iDv);
                du[o] = dun;
                dv[o] = dvn;
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_sor_global(const float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                              int n_frames, DiagGeom g, int G, float wa, float wb, float omega, cudaStream_t st)
{
    const int threads = g.h >= 1024 ? 1024 : ((g.h + 31) / 32) * 32;
    k_sor_global<<<n_frames, threads, 0, st>>>(coef, coef_fs, du, dv, st_fs, g, G, wa, wb, omega);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 5x5 median with scipy's "mirror" boundary on du and dv (core/optical_flow.py:
// 607-609), then u + du, v + dv on the interior (:610-611).
// The median is a forgetful selection: keep 14 candidates, repeatedly drop the
// minimum and maximum and admit the next value; the middle of the last three
// is the 13th smallest of the 25.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cswap(float& x, float& y)
{
    const float lo = fminf(x, y), hi = fmaxf(x, y);
    x = lo;
    y = hi;
}

__device__ __forceinline__ int mirror(int i, int n)
{
    // valid for n >= 3 and |offset| <= 2 beyond the edge
    if (i < 0) i = -i;
    if (i >= n) i = 2 * (n - 1) - i;
    return i;
}

__device__ float median25(float v[25])
{
    float t[14];
#pragma unroll
    for (int i = 0; i < 14; ++i) t[i] = v[i];
#pragma unroll
    for (int round = 0; round < 11; ++round) {
        const int lo = round;  // window t[lo..13]
#pragma unroll
        for (int i = lo + 1; i < 14; ++i) cswap(t[lo], t[i]);
#pragma unroll
        for (int i = lo + 1; i < 13; ++i) cswap(t[i], t[13]);
        t[13] = v[14 + round];
    }
    // window t[11..13]: median of three
    cswap(t[11], t[12]);
    cswap(t[12], t[13]);
    cswap(t[11], t[12]);
    return t[12];
}

__global__ void k_median_accum(const float* __restrict__ du, const float* __restrict__ dv, long long st_fs,
                               View u, View v, DiagGeom g, int do_median, ViewW out_u, ViewW out_v)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int f = blockIdx.z;
    if (x >= g.w) return;
    const float* duf = du + f * st_fs;
    const float* dvf = dv + f * st_fs;
    float mu, mv;
    if (do_median) {
        float a[25], b[25];
        int q = 0;
#pragma unroll
        for (int dy = -2; dy <= 2; ++dy) {
            const int yy = mirror(y + dy, g.h);
#pragma unroll
            for (int dx = -2; dx <= 2; ++dx) {
                const int xx = mirror(x + dx, g.w);
                const long long o = diag_index(g, yy, xx);
                a[q] = duf[o];
                b[q] = dvf[o];
                ++q;
            }
        }
        mu = median25(a);
        mv = median25(b);
    } else {
        const long long o = diag_index(g, y, x);
        mu = duf[o];
        mv = dvf[o];
    }
    const float uc = u.p[f * u.fs + (long long)(y + 1) * u.rs + (long long)(x + 1) * u.cs];
    const float vc = v.p[f * v.fs + (long long)(y + 1) * v.rs + (long long)(x + 1) * v.cs];
    out_u.p[f * out_u.fs + (long long)y * out_u.rs + (long long)x * out_u.cs] = uc + mu;
    out_v.p[f * out_v.fs + (long long)y * out_v.rs + (long long)x * out_v.cs] = vc + mv;
}

cudaError_t launch_median_accum(const float* du, const float* dv, long long st_fs, View u, View v,
                                int n_frames, DiagGeom g, int do_median, ViewW out_u, ViewW out_v,
                                cudaStream_t st)
{
    dim3 blk(128), grd((g.w + 127) / 128, g.h, n_frames);
    k_median_accum<<<grd, blk, 0, st>>>(du, dv, st_fs, u, v, g, do_median, out_u, out_v);
    return cudaGetLastError();
}

// Median + accumulate on row-major du, dv (T, h, w): a 32 x 16 output tile
// with its mirrored 2-pixel halo is staged in shared memory by coalesced row
// loads; each thread takes two vertically adjacent pixels, whose windows share
// four of their five rows (median25_pair).
constexpr int kMedTx = 32, kMedTy = 8, kMedRows = 2 * kMedTy;

__global__ void __launch_bounds__(kMedTx * kMedTy) k_median_rm(const float* __restrict__ du,
                                                               const float* __restrict__ dv, long long fs, View u,
                                                               View v, int h, int w, int do_median, ViewW out_u,
                                                               ViewW out_v)
{
    __shared__ float su[kMedRows + 4][kMedTx + 4];
    __shared__ float sv[kMedRows + 4][kMedTx + 4];
    const int f = blockIdx.z;
    const int x0 = blockIdx.x * kMedTx, y0 = blockIdx.y * kMedRows;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * kMedTx + tx;
    const float* duf = du + f * fs;
    const float* dvf = dv + f * fs;
    if (do_median) {
        for (int i = tid; i < (kMedRows + 4) * (kMedTx + 4); i += kMedTx * kMedTy) {
            const int r = i / (kMedTx + 4), c = i - r * (kMedTx + 4);
            const int yy = mirror(min(y0 - 2 + r, h + 1), h);
            const int xx = mirror(min(x0 - 2 + c, w + 1), w);
            su[r][c] = duf[(long long)yy * w + xx];
            sv[r][c] = dvf[(long long)yy * w + xx];
        }
        __syncthreads();
    }
    const int x = x0 + tx, ya = y0 + 2 * ty, yb = ya + 1;
    if (x >= w || ya >= h) return;
    float mua, mva, mub, mvb;
    if (do_median) {
        // window of ya: tile rows 2ty .. 2ty + 4; of yb: 2ty + 1 .. 2ty + 5
        float c20[20], ea[5], eb[5];
#pragma unroll
        for (int dy = 0; dy < 4; ++dy)
#pragma unroll
            for (int dx = 0; dx < 5; ++dx) c20[dy * 5 + dx] = su[2 * ty + 1 + dy][tx + dx];
#pragma unroll
        for (int dx = 0; dx < 5; ++dx) {
            ea[dx] = su[2 * ty][tx + dx];
            eb[dx] = su[2 * ty + 5][tx + dx];
        }
        median25_pair(c20, ea, eb, mua, mub);
#pragma unroll
        for (int dy = 0; dy < 4; ++dy)
#pragma unroll
            for (int dx = 0; dx < 5; ++dx) c20[dy * 5 + dx] = sv[2 * ty + 1 + dy][tx + dx];
#pragma unroll
        for (int dx = 0; dx < 5; ++dx) {
            ea[dx] = sv[2 * ty][tx + dx];
            eb[dx] = sv[2 * ty + 5][tx + dx];
        }
        median25_pair(c20, ea, eb, mva, mvb);
    } else {
        mua = duf[(long long)ya * w + x];
        mva = dvf[(long long)ya * w + x];
        mub = yb < h ? duf[(long long)yb * w + x] : 0.0f;
        mvb = yb < h ? dvf[(long long)yb * w + x] : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int y = ya + q;
        if (y >= h) break;
        const float uc = u.p[f * u.fs + (long long)(y + 1) * u.rs + (long long)(x + 1) * u.cs];
        const float vc = v.p[f * v.fs + (long long)(y + 1) * v.rs + (long long)(x + 1) * v.cs];
        out_u.p[f * out_u.fs + (long long)y * out_u.rs + (long long)x * out_u.cs] = uc + (q ? mub : mua);
        out_v.p[f * out_v.fs + (long long)y * out_v.rs + (long long)x * out_v.cs] = vc + (q ? mvb : mva);
    }
}

cudaError_t launch_median_rm(const float* du, const float* dv, long long fs, View u, View v, int n_frames, int h,
                             int w, int do_median, ViewW out_u, ViewW out_v, cudaStream_t st)
{
    dim3 blk(kMedTx, kMedTy), grd((w + kMedTx - 1) / kMedTx, (h + kMedRows - 1) / kMedRows, n_frames);
    k_median_rm<<<grd, blk, 0, st>>>(du, dv, fs, u, v, h, w, do_median, out_u, out_v);
    return cudaGetLastError();
}

}  // namespace frg
