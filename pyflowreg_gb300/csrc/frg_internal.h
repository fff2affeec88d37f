// Internal declarations shared by the CUDA kernels and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

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

// cudaFuncSetAttribute(cudaFuncAttributeMaxDynamicSharedMemorySize) holds per
// device: this sets it once per (kernel, current device) pair, so a process that
// launches on several GPUs gets it on each of them.  Thread-safe.
cudaError_t ensure_max_dyn_smem(const void* kernel, int bytes);
// Allows clusters of more than 8 CTAs for `kernel` on the current device (once).
cudaError_t ensure_nonportable_clusters(const void* kernel);

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
// launch_tensor plus the smoothness constant (launch_lap) from the same
// pixel tiles: one launch, both written diagonal-major in contiguous runs.
cudaError_t launch_tensor_lap(View f1, View f2, int n_frames, int K, int h, int w, float hy, float hx, int gray,
                              float* J, long long J_fs, DiagGeom g, View u, View v, float wx, float wy, float* lap,
                              long long lap_fs, cudaStream_t st);
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
                             float* out_dv = nullptr, long long out_fs = 0, int threads = 0);
// threads per CTA of launch_sor_fused: 0 = P (the rows of the level, rounded
// up to 32); otherwise a multiple of 32 in [P, 1024].
// The same pass with one thread per row and the state in registers (frg_sor.cu,
// k_sor_regs): levels of at most 512 (padded) rows, K <= 4, G <= kGMax; same
// arguments and bit-identical results.
bool sor_regs_supports(int K, const DiagGeom& g);
cudaError_t launch_sor_regs(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap,
                            long long lap_fs, float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                            int n_frames, int K, DiagGeom g, int G, int mode, int store_coef, const float* a_data,
                            float wx, float wy, float omega, cudaStream_t st, float* out_du = nullptr,
                            float* out_dv = nullptr, long long out_fs = 0);
// Every pass of a level in one launch of the rows-in-registers SOR (frg_sor.cu,
// k_sor_chain): a row starts its next pass as soon as it has finished the
// current one, so the passes follow each other without restarting the
// wavefront.  Pass p is the launch_sor_regs pass (G, mode, store_coef); the
// level's last pass writes out_du/out_dv when given.  Every level
// launch_sor_regs serves (levels over 512 rows as clusters of row strips),
// w >= 3, at most kMaxChain passes; bit-identical to one launch_sor_regs call
// per pass.
constexpr int kMaxChain = 64;
struct ChainPass {
    int G, mode, store_coef;
};
bool sor_chain_supports(int K, const DiagGeom& g, int n_passes);
cudaError_t launch_sor_chain(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap,
                             long long lap_fs, float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                             int n_frames, int K, DiagGeom g, const ChainPass* passes, int n_passes,
                             const float* a_data, float wx, float wy, float omega, cudaStream_t st,
                             float* out_du = nullptr, float* out_dv = nullptr, long long out_fs = 0);
// The float64 solver's power x^b for one exponent b with |b| <= 1 (frg_dpow.cuh,
// dpow_b): a table of 2^(e b) (1 / inv_j)^b as double-double over the top 20
// bits of a positive x (unbiased exponent e in [-17, 46], the top 8 fraction
// bits j), and the binomial series (1 + r)^b - 1 = b r + c2 r^2 + ... + c6 r^6.
constexpr int kPowEMin = -17;
constexpr int kPowTabN = 64 * 256;
struct PowTab64 {
    const double2* t = nullptr;  // kPowTabN entries on the device; null: the general power
    double c2 = 0.0, c3 = 0.0;
    float c4 = 0.0f, c5 = 0.0f, c6 = 0.0f;
};
// Host: fills tab (kPowTabN entries) and the series constants of *pt for
// exponent b (pt->t untouched); false, with nothing written, when |b| > 1.
bool make_pow_table(double b, double2* tab, PowTab64* pt);
// The chained SOR in float64 (frg_sor64.cu, k_sor_chain64): the schedule of
// launch_sor_chain with float64 state, coefficients and arithmetic (the parity
// precision).  J [6][K][D*P] (J11, J22, J33 + 1e-5, 2 J12, 2 J13, 2 J23), W
// [2][K][D*P] (W, then W * a_data), lap [2][D*P], coef [5][D*P] and the state
// du, dv [D*P] are diagonal-major doubles; the final pass writes du, dv
// at out + r * out_rs + c.  Levels of at most 2048 (padded) rows (over 256 as
// clusters of row strips), K <= 4, w >= 3, at most kMaxChain passes of G <= kGMax.
// rows: the most rows per CTA (64, 128 or 256; 0 = 256), the level split into at
// most 8 strips; every split gives the same bits.  pows: the power table of
// each channel's exponent a_data[k] - 1 (null, or a null table: the general
// power).
bool sor_chain64_supports(int K, const DiagGeom& g, int n_passes);
bool sor_chain64_rows_ok(const DiagGeom& g, int rows);
int sor_chain64_default_rows(const DiagGeom& g, int n_frames, int n_sms);
cudaError_t launch_sor_chain64(const double* J, long long J_fs, const double* W, long long W_fs, const double* lap,
                               long long lap_fs, double* coef, long long coef_fs, double* du, double* dv,
                               long long st_fs, int n_frames, int K, DiagGeom g, const ChainPass* passes,
                               int n_passes, const double* a_data, double wx, double wy, double omega,
                               cudaStream_t st, double* out_du, double* out_dv, long long out_fs, int out_rs,
                               int rows = 0, const PowTab64* pows = nullptr);
// x^b elementwise by the float64 solver's power (frg_dpow.cuh), with the table
// path for |b| <= 1; upload_dpow_tables must have run on the current device.
cudaError_t launch_pow64(long long n, const double* x, double b, double* out, cudaStream_t st);
cudaError_t upload_dpow_tables();
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
// The tensor diagonal-major (T, 6, K, D*P) with the smoothness constant
// (T, 2, D*P) from the padded float64 u, v (frame stride uv_fs), for the
// float64 chained SOR; f1 is the reference level in float64 (K, h, w) and rd
// its derivatives (launch_x_ref_derivs), f1f the same level in float32 (the
// census data term, gray = 2, runs the reference-order
// arithmetic of kx_tensor on it).  The planes hold J11, J22, J33 + 1e-5, 2 J12,
// 2 J13, 2 J23: the cross terms doubled (exact) and the offset of psi's argument
// (E + 1e-5) added to J33, as the solver's data residual uses them.
cudaError_t launch_x_tensor_diag(const double* f1, const double* rd, const float* f1f, const float* f2, int n_frames,
                                 int K, int h, int w, double hy, double hx, int f2_f32, int gray, double* J,
                                 long long J_fs, DiagGeom g, const double* u, const double* v, long long uv_fs,
                                 double wx, double wy, double* lap, long long lap_fs, cudaStream_t st);
// The reference level's derivatives that kx_tensor_diag reads (rd: planes
// (4, K, h, w) of gx1, gy1, fxx1, fyy1 of f1 (K, h, w) in float64, the same
// arithmetic as the tensor's), once per reference and level.
cudaError_t launch_x_ref_derivs(const double* f1, int K, int h, int w, double hy, double hx, double* rd,
                                cudaStream_t st);
cudaError_t launch_x_to_double(const float* src, long long n, double* dst, cudaStream_t st);
cudaError_t launch_x_sor(const double* J, const double* W, const double* u, const double* v, long long uv_fs,
                         double* du, double* dv, double* wp, int n_frames, int K, int h, int w, double alpha_x,
                         double alpha_y, double hx, double hy, int iterations, int update_lag,
                         const double* a_data, double omega, double gnc_beta, cudaStream_t st);
// a_smooth != 1: the SOR cut at the psi ticks (ticks recompute W psi and
// psi_s over the padded grid).  psi_s (T, m*n) and snap (T, 2, m*n) are
// workspace; *launches is incremented per kernel launched.  gnc_beta < 0: compute_flow;
// else compute_flow_gnc with that stage weight (both solvers).
cudaError_t launch_x_sor_smooth(const double* J, const double* W, const double* u, const double* v, long long uv_fs,
                                double* du, double* dv, double* wp, double* psi_s, double* snap, int n_frames, int K,
                                int h, int w, double alpha_x, double alpha_y, double hx, double hy, int iterations,
                                int update_lag, const double* a_data, double a_smooth, double omega, double gnc_beta,
                                cudaStream_t st, long long* launches);
cudaError_t launch_x_to_float(const double* src, long long n, float* dst, cudaStream_t st);
// Padded (K, (h+2)*(w+2)) float64 planes to diagonal-major (K, D*P).
// Padded (K, h + 2, w + 2) float64 planes to diagonal-major (K, D*P) at dst;
// with scale (K host values), also each plane times scale[k] at dst + K*D*P
// (the float64 chained SOR's weights W and W * a_data).
cudaError_t launch_x_pad_to_diag(const double* src, int K, int h, int w, DiagGeom g, double* dst, cudaStream_t st,
                                 const double* scale = nullptr);
cudaError_t launch_x_hwk_to_planes(const double* src, int n_arrays, long long mn, int K, double* dst, cudaStream_t st);
// cv2.resize INTER_CUBIC of planar planes (n_frames * n_planes, ih, iw) to
// (oh, ow): width pass into tmp, height pass into the strided dst view.
template <typename T>
cudaError_t launch_cubic_up(const T* src, int n_frames, int n_planes, int ih, int iw, T* tmp, T* dst, long long fs,
                            long long ps, long long rs, long long cs, int oh, int ow, const int32_t* sx,
                            const float* wx, const int32_t* sy, const float* wy, cudaStream_t st);
cudaError_t launch_x_median_accum(const double* du, const double* dv, const double* u, const double* v,
                                  long long uv_fs, int n_frames, int h, int w, int do_median, double* ou, double* ov,
                                  long long o_fs, long long o_rs, long long o_cs, cudaStream_t st);
// 5x5 median (mirror) of one float64 plane (h, w), h, w >= 3, by the kernel of
// launch_x_median_accum.
cudaError_t launch_x_median5_plane(const double* src, int h, int w, double* dst, cudaStream_t st);
// One GNC warping step's state update (two kernels, the second only when
// write_ring): (ou, ov) = [median5](u + du) interiors, then the padded u, v
// rebuilt from them.  Counts 1 + write_ring launches.
cudaError_t launch_x_gnc_update(const double* du, const double* dv, double* u, double* v, long long uv_fs,
                                int n_frames, int h, int w, int do_median, double* ou, double* ov, long long o_fs,
                                long long o_rs, long long o_cs, int write_ring, cudaStream_t st);

// Preprocessing and post-registration statistics (frg_prep.cu).
// taps w[k][0 .. r] stored with stride (max_k r + 1); radii per channel (host arrays)
cudaError_t launch_preprocess(const float* raw, const double* raw64, int T, int H, int W, int K, const double* lo,
                              const double* den, const double* wt, const int* rt, const double* wy, const int* ry,
                              const double* wx, const int* rx, int f32_norm, int f32_storage, void* tmp, float* out,
                              cudaStream_t st);
cudaError_t launch_flow_post(const float* flow, int T, int H, int W, uint8_t* valid, double* part, double* stats,
                             cudaStream_t st);

// Host helpers of frg_api.cu shared with the differentiable mode's C ABI
// (frg_diff_api.cu).
int host_fail(int code, const std::string& msg);
void host_count_launches(long long n);
int host_warping_depth(double eta, int levels, int m, int n);
double host_resize_sigma(int ih, int iw, int oh, int ow);
// Tap tables of the fused Gauss-cubic resize (util/resize_util.py:194-229).
int host_make_tables(int in_len, int out_len, double sigma, std::vector<int32_t>& idx, std::vector<float>& wt);

namespace diff {

// Inverse (CSR) form of a resize tap table: for each source index a, the
// entries ptr[a] .. ptr[a+1]-1 list the output indices idx[e] whose taps
// read a, with weight w[e].
struct Csr {
    const int32_t* ptr;
    const int32_t* idx;
    const float* w;
};

// Differentiable-mode launchers (frg_diff.cu), T = float or double.  Arrays
// are planar row-major: images (F, K, h, w), flows / solver states (F, 2, h, w),
// J (F, 6, K, h, w), coefficients (F, 5, h, w).
template <typename T>
cudaError_t resize(const T* src, long long planes, int ih, int iw, int oh, int ow, const int32_t* ix, const float* wx,
                   int Px, const int32_t* iy, const float* wy, int Py, T* tmp, T* dst, cudaStream_t st);
template <typename T>
cudaError_t resize_t(const T* gdst, long long planes, int oh, int ow, int ih, int iw, const Csr& cx, const Csr& cy,
                     T* tmp, T* gsrc, int accumulate, cudaStream_t st);
template <typename T>
cudaError_t warp(const T* f2, const T* f1, const T* uv, int F, int K, int h, int w, double hcol, double hrow, T* out,
                 cudaStream_t st);
template <typename T>
cudaError_t warp_adj(const T* f2, const T* uv, const T* gout, int F, int K, int h, int w, double hcol, double hrow,
                     T* gf2, T* gf1, T* guv, cudaStream_t st);
template <typename T>
cudaError_t tensor(const T* f1, const T* f2, int F, int K, int h, int w, double hy, double hx, T* J, cudaStream_t st);
template <typename T>
cudaError_t tensor_adj(const T* f1, const T* f2, const T* gJ, int F, int K, int h, int w, double hy, double hx, T* G,
                       T* gf1, T* gf2, int accumulate_f1, cudaStream_t st);
// Solver: coefficients (F, 5, h, w) = max(A11, eps), max(A22, eps), A12, B1e,
// B2e with the input flow's Laplacian folded into B1e, B2e.  States are full
// (F, 2, h, w) arrays; a half-sweep's moved pixels can also be stored
// compressed (F, 2, h, (w + 1) / 2).  gs = 1: dv of a moving pixel from its
// new du (numba's within-pixel order); gs = 0: from the old du (torch backend).
template <typename T>
cudaError_t tick(const T* J, const T* W, const T* stt, const T* uv, int F, int K, int h, int w, const double* a_data,
                 double eps, double ax, double ay, T* coef, T* ck, cudaStream_t st);
// rhs (F, 2, h, w) or NULL: with it the sweep solves M lam = rhs (B1e, B2e
// replaced by -rhs) for the level's symmetric operator M.
template <typename T>
cudaError_t rb_sweep(int color, const T* coef, const T* rhs, T* state, T* store, int F, int h, int w, double ax,
                     double ay, double omega, double eps, int gs, cudaStream_t st);
// Implicit adjoint assembly: gcoef (overwritten) and galpha from lam = M^-1 g
// and the level's final state x.
template <typename T>
cudaError_t implicit_assemble(const T* lam, const T* x, int F, int h, int w, T* gcoef, double sx, double sy,
                              double* galpha, cudaStream_t st);
// The adjoint kernels add their alpha gradients to per-block partial pairs
// (galpha arguments below): (F, h, ceil(n / 128), 2) doubles for a launch over
// n pixels of each row.  reduce_slots adds frame f's n_slots pairs to galpha
// (F, 2) and clears them.
cudaError_t reduce_slots(double* part, int F, long long n_slots, double* galpha, cudaStream_t st);
// Adjoint of half-sweep j (colour `color`) over the pixels it moves: first
// their gather of w * aprev (the (au, av) of step j + 1, compressed; NULL for
// the window's last half-sweep), then their own step, writing anext.  pre
// state: per colour a compressed array (pre_c0 / pre_c1) or, when that is
// NULL, the full array pre_full (NULL: zero).  galpha (F, 2) += (sx, sy) *
// d/d(ax, ay).  rb_adj_gather closes a window (the gather of step 0).
template <typename T>
cudaError_t rb_adj_step(int color, const T* coef, const T* pre_full, const T* pre_c0, const T* pre_c1, T* lam,
                        const T* aprev, T* anext, int F, int h, int w, double ax, double ay, double omega, double eps,
                        int gs, T* gcoef, double sx, double sy, double* galpha, cudaStream_t st);
template <typename T>
cudaError_t rb_adj_gather(int color, T* lam, const T* aprev, int F, int h, int w, double ax, double ay,
                          cudaStream_t st);
// All half-sweeps of one window in one launch (tiles with halos in shared
// memory): hist + j * slot holds the pixels half-sweep j moved, s0 the state
// before the window (NULL: zero); lam_in -> lam_out (distinct arrays), gcoef
// overwritten, galpha: one pair per CTA (F * ceil(h / tile) * ceil(w / tile)),
// summed by reduce_slots.  rb_adj_window_tile gives the tile edge for nh
// half-sweeps and an element size, 0 when the window does not fit.
constexpr size_t kAdjWindowSmem = 200 * 1024;
constexpr int kAdjMaxNh = 40;  // half-sweeps per window the tiled adjoint takes (update_lag <= 20)
// Ring tables of the tiled adjoint (device pointers per colour, counts per
// distance), built on the host by build_adj_table.
struct AdjTable {
    const int2* e[2];
    int cnt[2][kAdjMaxNh + 1];
};
bool build_adj_table(int tile, int nh, std::vector<int2>& e0, std::vector<int2>& e1, int cnt[2][kAdjMaxNh + 1]);
int rb_adj_window_tile(int nh, int elem_bytes);
template <typename T>
cudaError_t rb_adj_window(const T* coef, const T* s0, const T* hist, long long slot, const T* lam_in, T* lam_out,
                          int F, int h, int w, int nh, int tile, const AdjTable& tab, double ax, double ay,
                          double omega, double eps, int gs, T* gcoef, double sx, double sy, double* galpha,
                          cudaStream_t st);
template <typename T>
cudaError_t tick_adj(const T* J, const T* W, const T* stt, const T* uv, const T* gcoef, int F, int K, int h, int w,
                     const double* a_data, double eps, double ax, double ay, int lagged, T* gJ, T* lam, T* guv,
                     double sx, double sy, double* galpha, cudaStream_t st);
template <typename T>
cudaError_t median_add(const T* d, const T* uv_in, T* uv_out, int F, int h, int w, int median, cudaStream_t st);
template <typename T>
cudaError_t median_adj(const T* d, const T* g, int32_t* am, int F, int h, int w, T* gd, cudaStream_t st);
}  // namespace diff

}  // namespace frg
