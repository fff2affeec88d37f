// Per-frame work before and after the flow: input preprocessing and
// post-registration statistics, on the device.
//
// Preprocessing (motion_correction/compensate_recording.py:521-561,
// util/image_processing.py:12-165): normalisation by the raw reference's
// min/max ((x - lo) / (hi - lo + 1e-8), jointly or per channel), then a
// Gaussian filter per channel as scipy.ndimage.gaussian_filter applies it:
// one 1-D correlation per axis in axis order (time, rows, columns), mode
// "reflect" (d c b a | a b c d | d c b a), each output sum formed in double
// as scipy's symmetric correlation forms it (outermost pair first):
//   acc = x[i] * w[0];  for j = r .. 1:  acc += (x[i - j] + x[i + j]) * w[j]
// and stored in the input's precision after each pass: float32 when numpy
// keeps the normalised frames float32 (float32 frames and reference), float64
// otherwise.  The taps (w[0 .. r], normalised in float64 by the host) come
// from the caller.  The result is stored as float32, the type the flow path's
// resize consumes.
//
// Post-registration (motion_correction/compensate_recording.py:808-821,
// core/warping.py:14-60, 128-157): per frame the valid mask of the backward
// warp (x + u in [0, W), y + v in [0, H); 0 or 255), and the partial sums of
// |w|, max |w|, the divergence du/dx + dv/dy (np.gradient: central inside,
// one-sided at the edges), u and v, reduced per frame by a second kernel.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/flowreg_gb300.h"
#include "frg_internal.h"

namespace frg {

namespace {

__device__ __forceinline__ int reflect_scipy(int i, int n)
{
    // scipy.ndimage mode "reflect": the edge sample is repeated
    if (n == 1) return 0;
    const int period = 2 * n;
    i %= period;
    if (i < 0) i += period;
    return i < n ? i : period - 1 - i;
}

struct PrepArgs {
    const float* raw;   // (T, H, W, K) float32 frames, or
    const double* raw64;  // the same in float64 (then raw is NULL and numpy normalises in float64)
    int T, H, W, K;
    double lo[kMaxK], den[kMaxK];  // normalisation per channel (same value for all channels when joint)
    const double* wt;   // temporal taps [K][rt + 1] (channel k uses its first rtk[k] + 1)
    const double* wy;   // row taps [K][ry + 1]
    const double* wx;   // column taps [K][rx + 1]
    int rt, ry, rx;     // tap strides - 1 (the largest radius per axis)
    int rtk[kMaxK], ryk[kMaxK], rxk[kMaxK];  // radius per channel
};

// N: the precision numpy normalises in (float32 for float32 frames and
// reference, else float64); S: the storage of the normalised values and of
// every pass's output (N for joint normalisation; float64 for per-channel
// normalisation, which writes into a float64 array).  Sums are formed in
// double either way, as scipy's line buffers do.
template <typename S>
__device__ __forceinline__ S normed(const PrepArgs& A, int t, int y, int x, int k);
template <>
__device__ __forceinline__ float normed<float>(const PrepArgs& A, int t, int y, int x, int k)
{
    const float v = A.raw[(((long long)t * A.H + y) * A.W + x) * A.K + k];
    return __fdiv_rn(__fsub_rn(v, (float)A.lo[k]), (float)A.den[k]);
}
template <>
__device__ __forceinline__ double normed<double>(const PrepArgs& A, int t, int y, int x, int k)
{
    const long long i = (((long long)t * A.H + y) * A.W + x) * A.K + k;
    const double v = A.raw64 ? A.raw64[i] : (double)A.raw[i];
    return __ddiv_rn(__dsub_rn(v, A.lo[k]), A.den[k]);
}

// scipy's symmetric correlation of one output sample (no contraction):
// acc = c * w[0], then acc += (left_j + right_j) * w[j] for j = r .. 1
template <typename F>
__device__ __forceinline__ double corr_sym(const double* w, int r, double c, F at)
{
    double acc = __dmul_rn(c, w[0]);
    for (int j = r; j >= 1; --j) {
        double l, rr;
        at(j, l, rr);
        acc = __dadd_rn(acc, __dmul_rn(__dadd_rn(l, rr), w[j]));
    }
    return acc;
}

// value after the temporal pass, stored as S (the temporal pass is an
// identity, x * 1.0, when its radius is 0)
template <typename N, typename S>
__device__ __forceinline__ S tpass(const PrepArgs& A, int t, int y, int x, int k)
{
    const double* w = A.wt + (long long)k * (A.rt + 1);
    const double acc = corr_sym(w, A.rtk[k], (double)normed<N>(A, t, y, x, k), [&](int j, double& l, double& r) {
        l = (double)normed<N>(A, reflect_scipy(t - j, A.T), y, x, k);
        r = (double)normed<N>(A, reflect_scipy(t + j, A.T), y, x, k);
    });
    return (S)acc;
}

// pass 1: temporal and row correlation into tmp (T, K, H, W) of S
template <typename N, typename S>
__global__ void k_prep_rows(PrepArgs A, S* __restrict__ tmp)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= A.W) return;
    const int y = blockIdx.y;
    const int tk = blockIdx.z;
    const int t = tk / A.K, k = tk % A.K;
    const double* w = A.wy + (long long)k * (A.ry + 1);
    const double acc = corr_sym(w, A.ryk[k], (double)tpass<N, S>(A, t, y, x, k), [&](int j, double& l, double& r) {
        l = (double)tpass<N, S>(A, t, reflect_scipy(y - j, A.H), x, k);
        r = (double)tpass<N, S>(A, t, reflect_scipy(y + j, A.H), x, k);
    });
    tmp[((long long)tk * A.H + y) * A.W + x] = (S)acc;
}

// pass 2: column correlation; float32 output (T, H, W, K)
template <typename S>
__global__ void k_prep_cols(PrepArgs A, const S* __restrict__ tmp, float* __restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= A.W) return;
    const int y = blockIdx.y;
    const int tk = blockIdx.z;
    const int t = tk / A.K, k = tk % A.K;
    const S* row = tmp + ((long long)tk * A.H + y) * A.W;
    const double* w = A.wx + (long long)k * (A.rx + 1);
    const double acc = corr_sym(w, A.rxk[k], (double)row[x], [&](int j, double& l, double& r) {
        l = (double)row[reflect_scipy(x - j, A.W)];
        r = (double)row[reflect_scipy(x + j, A.W)];
    });
    out[(((long long)t * A.H + y) * A.W + x) * A.K + k] = (float)(S)acc;
}

// Post-registration pass over flows (T, H, W, 2): valid masks and per-block
// partials (sum |w|, max |w|, sum div, sum u, sum v) at part[(f, y, bx)][5].
__global__ void k_flow_post(const float* __restrict__ flow, int H, int W, uint8_t* __restrict__ valid,
                            double* __restrict__ part)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const long long f = blockIdx.z;
    double s_mag = 0, m_mag = 0, s_div = 0, s_u = 0, s_v = 0;
    if (x < W) {
        const float* w = flow + f * H * W * 2;
        const long long p = (long long)y * W + x;
        const float u = w[2 * p], v = w[2 * p + 1];
        const double mx = (double)x + (double)u, my = (double)y + (double)v;
        if (valid) valid[f * H * W + p] = (mx >= 0.0 && mx < (double)W && my >= 0.0 && my < (double)H) ? 255 : 0;
        const double mag = sqrt((double)u * u + (double)v * v);
        s_mag = mag;
        m_mag = mag;
        // np.gradient, edge_order 1
        double dudx, dvdy;
        if (W == 1) dudx = 0;
        else if (x == 0) dudx = (double)w[2 * (p + 1)] - u;
        else if (x == W - 1) dudx = u - (double)w[2 * (p - 1)];
        else dudx = ((double)w[2 * (p + 1)] - (double)w[2 * (p - 1)]) * 0.5;
        if (H == 1) dvdy = 0;
        else if (y == 0) dvdy = (double)w[2 * (p + W) + 1] - v;
        else if (y == H - 1) dvdy = v - (double)w[2 * (p - W) + 1];
        else dvdy = ((double)w[2 * (p + W) + 1] - (double)w[2 * (p - W) + 1]) * 0.5;
        s_div = dudx + dvdy;
        s_u = u;
        s_v = v;
    }
    __shared__ double red[5][256];
    const int t = threadIdx.x;
    red[0][t] = s_mag;
    red[1][t] = m_mag;
    red[2][t] = s_div;
    red[3][t] = s_u;
    red[4][t] = s_v;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (t < st) {
            red[0][t] += red[0][t + st];
            red[1][t] = fmax(red[1][t], red[1][t + st]);
            red[2][t] += red[2][t + st];
            red[3][t] += red[3][t + st];
            red[4][t] += red[4][t + st];
        }
        __syncthreads();
    }
    if (t == 0) {
        double* o = part + (((f * gridDim.y + y) * gridDim.x) + blockIdx.x) * 5;
        for (int q = 0; q < 5; ++q) o[q] = red[q][0];
    }
}

// stats (T, 4): mean |w|, max |w|, mean divergence, |mean w|
__global__ void k_flow_stats(const double* __restrict__ part, long long n_slots, double n_pix, double* __restrict__ stats)
{
    const long long f = blockIdx.x;
    const double* p = part + f * n_slots * 5;
    double a = 0, m = 0, d = 0, su = 0, sv = 0;
    for (long long i = threadIdx.x; i < n_slots; i += blockDim.x) {
        a += p[5 * i];
        m = fmax(m, p[5 * i + 1]);
        d += p[5 * i + 2];
        su += p[5 * i + 3];
        sv += p[5 * i + 4];
    }
    __shared__ double red[5][256];
    const int t = threadIdx.x;
    red[0][t] = a;
    red[1][t] = m;
    red[2][t] = d;
    red[3][t] = su;
    red[4][t] = sv;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (t < st) {
            red[0][t] += red[0][t + st];
            red[1][t] = fmax(red[1][t], red[1][t + st]);
            red[2][t] += red[2][t + st];
            red[3][t] += red[3][t + st];
            red[4][t] += red[4][t + st];
        }
        __syncthreads();
    }
    if (t == 0) {
        const double mu = red[3][0] / n_pix, mv = red[4][0] / n_pix;
        stats[4 * f] = red[0][0] / n_pix;
        stats[4 * f + 1] = red[1][0];
        stats[4 * f + 2] = red[2][0] / n_pix;
        stats[4 * f + 3] = sqrt(mu * mu + mv * mv);
    }
}

}  // namespace

cudaError_t launch_preprocess(const float* raw, const double* raw64, int T, int H, int W, int K, const double* lo,
                              const double* den, const double* wt, const int* rt, const double* wy, const int* ry,
                              const double* wx, const int* rx, int f32_norm, int f32_storage, void* tmp, float* out,
                              cudaStream_t st)
{
    PrepArgs A;
    A.raw = raw;
    A.raw64 = raw64;
    A.T = T;
    A.H = H;
    A.W = W;
    A.K = K;
    for (int k = 0; k < kMaxK; ++k) {
        A.lo[k] = k < K ? lo[k] : 0.0;
        A.den[k] = k < K ? den[k] : 1.0;
    }
    A.wt = wt;
    A.wy = wy;
    A.wx = wx;
    A.rt = A.ry = A.rx = 0;
    for (int k = 0; k < kMaxK; ++k) {
        A.rtk[k] = k < K ? rt[k] : 0;
        A.ryk[k] = k < K ? ry[k] : 0;
        A.rxk[k] = k < K ? rx[k] : 0;
        A.rt = A.rtk[k] > A.rt ? A.rtk[k] : A.rt;
        A.ry = A.ryk[k] > A.ry ? A.ryk[k] : A.ry;
        A.rx = A.rxk[k] > A.rx ? A.rxk[k] : A.rx;
    }
    const dim3 grid((unsigned)((W + 127) / 128), (unsigned)H, (unsigned)(T * K));
    if (f32_storage) {
        k_prep_rows<float, float><<<grid, 128, 0, st>>>(A, (float*)tmp);
        k_prep_cols<float><<<grid, 128, 0, st>>>(A, (const float*)tmp, out);
    } else if (f32_norm) {
        k_prep_rows<float, double><<<grid, 128, 0, st>>>(A, (double*)tmp);
        k_prep_cols<double><<<grid, 128, 0, st>>>(A, (const double*)tmp, out);
    } else {
        k_prep_rows<double, double><<<grid, 128, 0, st>>>(A, (double*)tmp);
        k_prep_cols<double><<<grid, 128, 0, st>>>(A, (const double*)tmp, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_flow_post(const float* flow, int T, int H, int W, uint8_t* valid, double* part, double* stats,
                             cudaStream_t st)
{
    const dim3 grid((unsigned)((W + 255) / 256), (unsigned)H, (unsigned)T);
    k_flow_post<<<grid, 256, 0, st>>>(flow, H, W, valid, part);
    k_flow_stats<<<T, 256, 0, st>>>(part, (long long)H * grid.x, (double)H * W, stats);
    return cudaGetLastError();
}

}  // namespace frg

extern "C" {

namespace {

int preprocess_checked(int n_frames, int height, int width, int channels, const float* raw, const double* raw64,
                       const double* lo, const double* den, const double* wt, const int* rt, const double* wy,
                       const int* ry, const double* wx, const int* rx, int f32_norm, int f32_storage, void* tmp,
                       float* out, void* stream)
{
    using namespace frg;
    if ((!raw && !raw64) || !lo || !den || !wt || !wy || !wx || !rt || !ry || !rx || !tmp || !out)
        return host_fail(FRG_EINVAL, "NULL argument");
    if (n_frames < 1 || height < 1 || width < 1 || channels < 1 || channels > kMaxK)
        return host_fail(FRG_EINVAL, "bad shape");
    if ((long long)n_frames * channels > 65535 || height > 65535) return host_fail(FRG_EINVAL, "batch too large");
    for (int k = 0; k < channels; ++k)
        if (rt[k] < 0 || ry[k] < 0 || rx[k] < 0) return host_fail(FRG_EINVAL, "negative filter radius");
    if (f32_storage && !f32_norm) return host_fail(FRG_EINVAL, "float32 storage needs float32 normalisation");
    if (raw64 && f32_norm) return host_fail(FRG_EINVAL, "float64 frames normalise in float64");
    for (int k = 0; k < channels; ++k)
        if (!(den[k] != 0.0)) return host_fail(FRG_EINVAL, "zero normalisation range");
    host_count_launches(2);
    cudaError_t e = launch_preprocess(raw, raw64, n_frames, height, width, channels, lo, den, wt, rt, wy, ry, wx, rx,
                                      f32_norm, f32_storage, tmp, out, (cudaStream_t)stream);
    if (e != cudaSuccess) return host_fail(FRG_ECUDA, cudaGetErrorString(e));
    return FRG_OK;
}

}  // namespace

int frg_preprocess(int n_frames, int height, int width, int channels, const float* raw, const double* lo,
                   const double* den, const double* wt, const int* rt, const double* wy, const int* ry,
                   const double* wx, const int* rx, int f32_norm, int f32_storage, void* tmp, float* out, void* stream)
{
    if (!raw) return frg::host_fail(FRG_EINVAL, "NULL argument");
    return preprocess_checked(n_frames, height, width, channels, raw, nullptr, lo, den, wt, rt, wy, ry, wx, rx,
                              f32_norm, f32_storage, tmp, out, stream);
}

int frg_preprocess_f64(int n_frames, int height, int width, int channels, const double* raw, const double* lo,
                       const double* den, const double* wt, const int* rt, const double* wy, const int* ry,
                       const double* wx, const int* rx, int f32_storage, void* tmp, float* out, void* stream)
{
    if (!raw) return frg::host_fail(FRG_EINVAL, "NULL argument");
    return preprocess_checked(n_frames, height, width, channels, nullptr, raw, lo, den, wt, rt, wy, ry, wx, rx, 0,
                              f32_storage, tmp, out, stream);
}

size_t frg_flow_post_workspace(int n_frames, int height, int width)
{
    return (size_t)n_frames * height * ((width + 255) / 256) * 5 * sizeof(double);
}

int frg_flow_post(int n_frames, int height, int width, const float* flow, unsigned char* valid, void* workspace,
                  double* stats, void* stream)
{
    using namespace frg;
    if (!flow || !workspace || !stats) return host_fail(FRG_EINVAL, "NULL argument");
    if (n_frames < 1 || n_frames > 65535 || height < 1 || height > 65535 || width < 1)
        return host_fail(FRG_EINVAL, "bad shape");
    host_count_launches(2);
    cudaError_t e = launch_flow_post(flow, n_frames, height, width, valid, (double*)workspace, stats,
                                     (cudaStream_t)stream);
    if (e != cudaSuccess) return host_fail(FRG_ECUDA, cudaGetErrorString(e));
    return FRG_OK;
}

}  // extern "C"

