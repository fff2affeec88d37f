// Internal declarations shared by the CUDA kernels and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace frg {

constexpr int kMaxK = 8;        // channels per frame handled by one plan
constexpr int kGMax = 5;        // SOR iterations pipelined per wavefront pass
constexpr int kMaxLane = 512;   // longest diagonal (rows of the level) per CTA
constexpr int kRing = 2 * kGMax + 2;
constexpr int kPrefetch = 4;    // diagonals loaded ahead into registers

// 2-D strided view of a stack of planes: element (frame, plane, y, x) at
// base + frame*fs + plane*ps + y*rs + x*cs (all in elements).
struct View {
    const float* p;
    long long fs, ps, rs, cs;
};
struct ViewW {
    float* p;
    long long fs, ps, rs, cs;
};

// Diagonal-major layout of an h x w level interior: pixel (r, c) lives at
// (r + c) * P + r, P = h rounded up to 32.  One diagonal is contiguous, so a
// warp reading consecutive rows of one diagonal issues one 128-byte access.
struct DiagGeom {
    int h, w, D, P;
};

__host__ __device__ inline long long diag_index(const DiagGeom& g, int r, int c)
{
    return (long long)(r + c) * g.P + r;
}

// Kernel launchers (frg_kernels.cu).  All enqueue on `st` and return the
// launch status; none synchronises.
cudaError_t launch_resize_h(View src, int n_frames, int n_planes, int ih, int iw, float* dst, int ow,
                            const int32_t* ix, const float* wx, int P, cudaStream_t st);
cudaError_t launch_resize_v(const float* src, int n_frames, int n_planes, int ih, int ow, ViewW dst,
                            int oh, int pad, const int32_t* iy, const float* wy, int P, cudaStream_t st);
cudaError_t launch_warp(View f2, View f1, View u, View v, int n_frames, int K, int h, int w,
                        float h_col, float h_row, int cubic, ViewW out, cudaStream_t st);
cudaError_t launch_tensor(View f1, View f2, int n_frames, int K, int h, int w, float hy, float hx,
                          int gray, float* J, long long J_fs, DiagGeom g, cudaStream_t st);
cudaError_t launch_lap(View u, View v, int n_frames, int h, int w, float wx, float wy, float* lap,
                       long long lap_fs, DiagGeom g, cudaStream_t st);
cudaError_t launch_to_diag(View src, int n_frames, int n_planes, int h, int w, float* dst,
                           long long dst_fs, DiagGeom g, cudaStream_t st);
cudaError_t launch_from_diag(const float* src, long long src_fs, int n_frames, int n_planes, DiagGeom g,
                             ViewW dst, int ring, int ring_mode, cudaStream_t st);
cudaError_t launch_fold(const float* J, long long J_fs, const float* W, long long W_fs,
                        const float* lap, long long lap_fs, float* du, float* dv,
                        long long st_fs, float* coef, long long coef_fs, int n_frames, int K,
                        DiagGeom g, const float* a_data, int mode, float wx, float wy,
                        cudaStream_t st);
cudaError_t launch_sor(const float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                       int n_frames, DiagGeom g, int G, float wa, float wb, float omega,
                       cudaStream_t st);
// Pass on global memory for levels of any height (coefficients from the fold kernel).
cudaError_t launch_sor_global(const float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                              int n_frames, DiagGeom g, int G, float wa, float wb, float omega, cudaStream_t st);
// Largest pass length the fused kernel's shared-memory ring allows for a level
// of P (padded) rows; 0 when the level is too tall for it.
int sor_fused_gmax(int P);
// SOR with the fold in its loader (frg_sor.cu), K <= 4.  mode: -1 reads the
// coefficients stored by the group's first pass; else bit0 du = dv = 0, bit1
// psi tick.  store_coef writes the folded coefficients for continuation passes.
bool sor_fused_supports(int K);
// out_du/out_dv (optional, frame stride out_fs): the pass writes its result
// row-major (h, w) there instead of back into du/dv (the level's last pass).
cudaError_t launch_sor_fused(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap,
                             long long lap_fs, float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                             int n_frames, int K, DiagGeom g, int G, int mode, int store_coef, const float* a_data,
                             float wx, float wy, float omega, cudaStream_t st, float* out_du = nullptr,
                             float* out_dv = nullptr, long long out_fs = 0);
// 5x5 median (mirror) of row-major du, dv (T, h, w) plus accumulation into u, v.
cudaError_t launch_median_rm(const float* du, const float* dv, long long fs, View u, View v, int n_frames, int h,
                             int w, int do_median, ViewW out_u, ViewW out_v, cudaStream_t st);
cudaError_t launch_median_accum(const float* du, const float* dv, long long st_fs, View u, View v,
                                int n_frames, DiagGeom g, int do_median, ViewW out_u, ViewW out_v,
                                cudaStream_t st);
cudaError_t upload_cubic_table(const float* tab128, const float* lin64);

// FP64 reference-order kernels (frg_exact.cu).
cudaError_t upload_cubic_table_x(const float* tab128);
cudaError_t launch_x_resize_h_f(const float* src, long long fs, long long ps, long long rs, long long cs,
                                int n_frames, int n_planes, int ih, float* dst, int ow, const int32_t* ix,
                                const float* wx, int P, cudaStream_t st);
cudaError_t launch_x_resize_h_d(const double* src, long long fs, long long ps, long long rs, long long cs,
                                int n_frames, int n_planes, int ih, float* dst, int ow, const int32_t* ix,
                                const float* wx, int P, cudaStream_t st);
cudaError_t launch_x_resize_v_f(const float* src, int n_frames, int n_planes, int ih, int ow, float* dst,
                                long long fs, long long ps, long long rs, int oh, int ring, const int32_t* iy,
                                const float* wy, int P, cudaStream_t st);
cudaError_t launch_x_resize_v_d(const float* src, int n_frames, int n_planes, int ih, int ow, double* dst,
                                long long fs, long long ps, long long rs, int oh, int ring, const int32_t* iy,
                                const float* wy, int P, cudaStream_t st);
cudaError_t launch_x_warp(const float* f2, const float* f1, const double* u, const double* v, long long uv_fs,
                          int n_frames, int K, int h, int w, double h_col, double h_row, float* out, cudaStream_t st);
cudaError_t launch_x_tensor(const float* f1, const float* f2, int n_frames, int K, int h, int w, double hy, double hx,
                            int f2_f32, int gray, double* J, cudaStream_t st);
cudaError_t launch_x_sor(const double* J, const double* W, const double* u, const double* v, long long uv_fs,
                         double* du, double* dv, double* wp, int n_frames, int K, int h, int w, double alpha_x,
                         double alpha_y, double hx, double hy, int iterations, int update_lag,
                         const double* a_data, double omega, cudaStream_t st);
// cv2.resize INTER_CUBIC of planar planes (n_frames * n_planes, ih, iw) to
// (oh, ow): width pass into tmp, height pass into the strided dst view.
template <typename T>
cudaError_t launch_cubic_up(const T* src, int n_frames, int n_planes, int ih, int iw, T* tmp, T* dst, long long fs,
                            long long ps, long long rs, long long cs, int oh, int ow, const int32_t* sx,
                            const float* wx, const int32_t* sy, const float* wy, cudaStream_t st);
cudaError_t launch_x_median_accum(const double* du, const double* dv, const double* u, const double* v,
                                  long long uv_fs, int n_frames, int h, int w, int do_median, double* ou, double* ov,
                                  long long o_fs, long long o_rs, long long o_cs, cudaStream_t st);

}  // namespace frg
