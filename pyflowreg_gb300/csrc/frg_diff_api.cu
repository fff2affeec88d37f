// C ABI of the differentiable mode: plan, checkpointed forward, adjoint.
//
// Forward (frg_diff_forward), per level from coarse to fine, as
// _solve_displacement_stage (core/optical_flow.py:476-617) with the torch
// backend's solver (torch/core/level_solver.py:11-199):
//   f1, f2 = resize(fixed), resize(moving)         -> checkpoint
//   u, v   = resize(previous level's flow)         -> checkpoint
//   f2w    = warp(f2, u, v) (not at the top level)
//   J      = motion tensor(f1, f2w)
//   du, dv = red-black lagged-psi SOR; the state at every psi tick -> checkpoint
//   u, v  += median5(du), median5(dv)
// Backward (frg_diff_backward), per level from fine to coarse: recompute f2w
// and J from the checkpoints; for each tick window from the last to the first,
// recompute the tick's coefficients, re-run the window's half-sweeps from its
// checkpointed state keeping the pixels each one moves (or, with
// FRG_DIFF_STORE_SWEEPS, read them as the forward stored them), then run the
// half-sweeps' adjoints in reverse and the tick's adjoint; then the tensor,
// warp and resize adjoints.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/flowreg_gb300.h"
#include "frg_internal.h"

using namespace frg;

namespace {

#define DCUDA(call)                                                                           \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return host_fail(FRG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

// Counts the kernels a launcher enqueues (frg_launch_count) and checks it.
#define DLAUNCH(n, call)              \
    do {                              \
        host_count_launches(n);       \
        DCUDA(call);                  \
    } while (0)

constexpr double kEps = 1e-6;  // torch/core/level_solver.py:28

// Forward taps of one resize (out_w x P, out_h x P) and their inverse tables.
struct DTab {
    int P = 0;
    int in_h = 0, in_w = 0, out_h = 0, out_w = 0;
    int32_t* ix = nullptr;
    float* wx = nullptr;
    int32_t* iy = nullptr;
    float* wy = nullptr;
    int32_t* xptr = nullptr;
    int32_t* xidx = nullptr;
    float* xw = nullptr;
    int32_t* yptr = nullptr;
    int32_t* yidx = nullptr;
    float* yw = nullptr;
};

struct DLevel {
    int i = 0, h = 0, w = 0;
    bool top = false;
    double h_row = 1, h_col = 1, scale = 1;
    int sh = 0, sw = 0;  // flow source size
    DTab img, flow;
    void* Wl = nullptr;        // (K, h, w)
    void* ck_f1 = nullptr;     // (F, K, h, w)
    void* ck_f2 = nullptr;     // (F, K, h, w)
    void* ck_uv = nullptr;     // (F, 2, h, w): the level's input flow
    void* ck_ticks = nullptr;  // (n_ticks - 1, F, 2, h, w)
    void* ck_sweeps = nullptr; // FRG_DIFF_STORE_SWEEPS: (2 * iterations, F, 2, h, (w + 1) / 2)
    void* ck_final = nullptr;  // FRG_DIFF_STORE_SWEEPS: (F, 2, h, w), the level's final du, dv
    void* ck_coef = nullptr;   // FRG_DIFF_STORE_SWEEPS: (n_ticks, F, 5, h, w), each tick window's coefficients
    double ax = 0, ay = 0;     // smoothness weights of the last forward
};

// Inverse of a tap table: rows of the source index, entries (output index, weight).
void invert(const std::vector<int32_t>& idx, const std::vector<float>& wt, int P, int out_len, int in_len,
            std::vector<int32_t>& ptr, std::vector<int32_t>& oidx, std::vector<float>& ow)
{
    ptr.assign(in_len + 1, 0);
    for (int o = 0; o < out_len; ++o)
        for (int t = 0; t < P; ++t) ++ptr[idx[(size_t)o * P + t] + 1];
    for (int a = 0; a < in_len; ++a) ptr[a + 1] += ptr[a];
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    oidx.assign((size_t)out_len * P, 0);
    ow.assign((size_t)out_len * P, 0.0f);
    for (int o = 0; o < out_len; ++o)
        for (int t = 0; t < P; ++t) {
            const int a = idx[(size_t)o * P + t];
            oidx[fill[a]] = o;
            ow[fill[a]] = wt[(size_t)o * P + t];
            ++fill[a];
        }
}

}  // namespace

struct frg_diff_plan {
    frg_params p{};
    int H = 0, W = 0, K = 0, maxF = 0;
    bool dbl = false;
    size_t es = 4;
    int n_ticks = 0, win = 0;
    int gs = 1;  // within-pixel order: 1 dv from the new du (numba), 0 from the old (torch backend)
    bool store_sweeps = false;
    double a_data[kMaxK] = {0};
    std::vector<DLevel> levels;
    std::vector<void*> allocs;
    size_t bytes = 0;
    bool has_weight = false;
    int last_F = 0;
    bool have_forward = false;
    double alpha_x = 0, alpha_y = 0;
    // workspace
    void* tmp = nullptr;     // (F, max(K, 2), H, W)
    void* f2w = nullptr;     // (F, K, hw)
    void* J = nullptr;       // (F, 6, K, hw)
    void* coef = nullptr;    // (F, 5, hw)
    void* st = nullptr;      // (F, 2, hw)
    void* uvc[2] = {nullptr, nullptr};
    void* states = nullptr;  // (2 * win, F, 2, h, (w + 1) / 2): moved pixels of a window's half-sweeps
    void* lam[2] = {nullptr, nullptr};
    void* abuf[2] = {nullptr, nullptr};  // (F, 2, h, (w + 1) / 2): (au, av) of a half-sweep's moving pixels
    void* gcoef = nullptr;   // (F, 5, hw)
    void* guv = nullptr;     // (F, 2, hw)
    void* galpha = nullptr;  // (F, 2) doubles, when the caller passes none
    double* partA = nullptr; // per-block alpha partials of the half-sweep adjoints (F, H, ceil(ceil(W/2)/128), 2)
    double* partB = nullptr; // per-block alpha partials of the per-pixel adjoints (F, H, ceil(W/128), 2)
    double* partC = nullptr; // per-tile alpha partials of the tiled window adjoints (F, ceil(H/16), ceil(W/16), 2)
    // tiled window adjoint: tile edge (0: stepwise only) and the ring tables of
    // the full window and of a shorter last window
    int adj_tile = 0;
    int adj_nh[2] = {0, 0};
    frg::diff::AdjTable adj_tab[2];
    void* gJ = nullptr;      // (F, 6, K, hw)
    void* G = nullptr;       // (F, K, 5, hw)
    void* gf1 = nullptr;     // (F, K, hw)
    void* gf2w = nullptr;    // (F, K, hw)
    void* gf2l = nullptr;    // (F, K, hw)
    void* gout[2] = {nullptr, nullptr};
    int32_t* am = nullptr;   // (F, 2, hw)
};

namespace {

int dalloc(frg_diff_plan* pl, void** out, size_t bytes)
{
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return host_fail(FRG_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    pl->allocs.push_back(p);
    pl->bytes += bytes;
    *out = p;
    return FRG_OK;
}

template <typename P>
int dalloc_t(frg_diff_plan* pl, P** out, size_t count)
{
    void* p = nullptr;
    int rc = dalloc(pl, &p, count * sizeof(P));
    *out = (P*)p;
    return rc;
}

// The tiled window adjoint's tile edge and ring tables, for the full tick
// window and for a shorter last one (when iterations is not a multiple of
// update_lag); none when the window does not fit (the backward then runs
// stepwise).
int make_adj_tables(frg_diff_plan* pl)
{
    const int nh_full = 2 * pl->win;
    const int I = pl->p.iterations, lag = pl->p.update_lag;
    const int nh_last = 2 * (I - (pl->n_ticks - 1) * lag);
    const int tile = nh_full <= frg::diff::kAdjMaxNh ? frg::diff::rb_adj_window_tile(nh_full, (int)pl->es) : 0;
    if (!tile) return FRG_OK;
    const int nhs[2] = {nh_full, nh_last};
    for (int q = 0; q < 2; ++q) {
        if (q == 1 && nh_last == nh_full) {
            pl->adj_nh[1] = nh_full;
            pl->adj_tab[1] = pl->adj_tab[0];
            break;
        }
        std::vector<int2> e0, e1;
        frg::diff::AdjTable& tb = pl->adj_tab[q];
        if (!frg::diff::build_adj_table(tile, nhs[q], e0, e1, tb.cnt)) return FRG_OK;
        void* d = nullptr;
        int rc = dalloc(pl, &d, (e0.size() + e1.size()) * sizeof(int2));
        if (rc != FRG_OK) return rc;
        cudaError_t e = cudaMemcpy(d, e0.data(), e0.size() * sizeof(int2), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy((int2*)d + e0.size(), e1.data(), e1.size() * sizeof(int2), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return host_fail(FRG_ECUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        tb.e[0] = (const int2*)d;
        tb.e[1] = (const int2*)d + e0.size();
        pl->adj_nh[q] = nhs[q];
    }
    pl->adj_tile = tile;
    return FRG_OK;
}

// Uploads forward tables (ix/wx over out_w, iy/wy over out_h) and their inverses.
int put_tables(frg_diff_plan* pl, DTab* d, const int32_t* ix, const float* wx, const int32_t* iy, const float* wy)
{
    const size_t nx = (size_t)d->out_w * d->P, ny = (size_t)d->out_h * d->P;
    std::vector<int32_t> vix(ix, ix + nx), viy(iy, iy + ny);
    std::vector<float> vwx(wx, wx + nx), vwy(wy, wy + ny);
    std::vector<int32_t> xptr, xidx, yptr, yidx;
    std::vector<float> xw, yw;
    invert(vix, vwx, d->P, d->out_w, d->in_w, xptr, xidx, xw);
    invert(viy, vwy, d->P, d->out_h, d->in_h, yptr, yidx, yw);
    int rc;
    if (!d->ix) {
        if ((rc = dalloc_t(pl, &d->ix, nx)) || (rc = dalloc_t(pl, &d->wx, nx)) || (rc = dalloc_t(pl, &d->iy, ny)) ||
            (rc = dalloc_t(pl, &d->wy, ny)) || (rc = dalloc_t(pl, &d->xptr, xptr.size())) ||
            (rc = dalloc_t(pl, &d->xidx, nx)) || (rc = dalloc_t(pl, &d->xw, nx)) ||
            (rc = dalloc_t(pl, &d->yptr, yptr.size())) || (rc = dalloc_t(pl, &d->yidx, ny)) ||
            (rc = dalloc_t(pl, &d->yw, ny)))
            return rc;
    }
    DCUDA(cudaMemcpy(d->ix, vix.data(), nx * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->wx, vwx.data(), nx * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->iy, viy.data(), ny * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->wy, vwy.data(), ny * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->xptr, xptr.data(), xptr.size() * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->xidx, xidx.data(), nx * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->xw, xw.data(), nx * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->yptr, yptr.data(), yptr.size() * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->yidx, yidx.data(), ny * 4, cudaMemcpyHostToDevice));
    DCUDA(cudaMemcpy(d->yw, yw.data(), ny * 4, cudaMemcpyHostToDevice));
    return FRG_OK;
}

int make_dtab(frg_diff_plan* pl, DTab* d, int in_h, int in_w, int out_h, int out_w)
{
    d->in_h = in_h;
    d->in_w = in_w;
    d->out_h = out_h;
    d->out_w = out_w;
    const double sig = host_resize_sigma(in_h, in_w, out_h, out_w);
    std::vector<int32_t> ix, iy;
    std::vector<float> wx, wy;
    d->P = host_make_tables(in_w, out_w, sig, ix, wx);
    host_make_tables(in_h, out_h, sig, iy, wy);
    return put_tables(pl, d, ix.data(), wx.data(), iy.data(), wy.data());
}

diff::Csr csr_x(const DTab& d) { return diff::Csr{d.xptr, d.xidx, d.xw}; }
diff::Csr csr_y(const DTab& d) { return diff::Csr{d.yptr, d.yidx, d.yw}; }

template <typename T>
int run_forward(frg_diff_plan* pl, int F, const T* fixed, const T* moving, const T* uv_init, T* flow_out,
                cudaStream_t st)
{
    using namespace frg::diff;
    const int K = pl->K, H = pl->H, W = pl->W;
    const int I = pl->p.iterations, lag = pl->p.update_lag;
    const double om = pl->p.omega;
    T* tmp = (T*)pl->tmp;
    int cur = 0;
    const DLevel* prev = nullptr;
    for (DLevel& L : pl->levels) {
        const int h = L.h, w = L.w;
        const long long hw = (long long)h * w;
        T* f1 = (T*)L.ck_f1;
        T* f2 = (T*)L.ck_f2;
        T* uv = (T*)L.ck_uv;
        DLAUNCH(2, resize<T>(fixed, (long long)F * K, H, W, h, w, L.img.ix, L.img.wx, L.img.P, L.img.iy, L.img.wy,
                             L.img.P, tmp, f1, st));
        DLAUNCH(2, resize<T>(moving, (long long)F * K, H, W, h, w, L.img.ix, L.img.wx, L.img.P, L.img.iy, L.img.wy,
                             L.img.P, tmp, f2, st));
        if (L.top) {
            if (uv_init)
                DLAUNCH(2, resize<T>(uv_init, (long long)F * 2, H, W, h, w, L.flow.ix, L.flow.wx, L.flow.P,
                                     L.flow.iy, L.flow.wy, L.flow.P, tmp, uv, st));
            else
                DCUDA(cudaMemsetAsync(uv, 0, (size_t)F * 2 * hw * sizeof(T), st));
        } else {
            DLAUNCH(2, resize<T>((const T*)pl->uvc[cur], (long long)F * 2, prev->h, prev->w, h, w, L.flow.ix,
                                 L.flow.wx, L.flow.P, L.flow.iy, L.flow.wy, L.flow.P, tmp, uv, st));
        }
        const T* f2w = f2;
        if (!L.top) {
            DLAUNCH(1, warp<T>(f2, f1, uv, F, K, h, w, L.h_col, L.h_row, (T*)pl->f2w, st));
            f2w = (const T*)pl->f2w;
        }
        T* J = (T*)pl->J;
        T* coef = (T*)pl->coef;
        DLAUNCH(1, tensor<T>(f1, f2w, F, K, h, w, L.h_row, L.h_col, J, st));
        L.ax = (pl->alpha_x * L.scale) / (L.h_col * L.h_col);
        L.ay = (pl->alpha_y * L.scale) / (L.h_row * L.h_row);
        T* s = (T*)pl->st;
        DCUDA(cudaMemsetAsync(s, 0, (size_t)F * 2 * hw * sizeof(T), st));
        const size_t slot = (size_t)F * 2 * h * ((w + 1) / 2);
        for (int it = 0; it < I; ++it) {
            if (it % lag == 0) {
                const int k = it / lag;
                T* ck = k > 0 ? (T*)L.ck_ticks + (size_t)(k - 1) * F * 2 * hw : nullptr;
                // with stored sweeps each window's coefficients are kept too (the backward reads them)
                coef = pl->store_sweeps ? (T*)L.ck_coef + (size_t)k * F * 5 * hw : (T*)pl->coef;
                DLAUNCH(1, tick<T>(J, (const T*)L.Wl, k > 0 ? s : (const T*)nullptr, uv, F, K, h, w, pl->a_data, kEps,
                                   L.ax, L.ay, coef, ck, st));
            }
            for (int c = 0; c < 2; ++c) {
                T* store = pl->store_sweeps ? (T*)L.ck_sweeps + (size_t)(2 * it + c) * slot : nullptr;
                DLAUNCH(1, rb_sweep<T>(c, coef, (const T*)nullptr, s, store, F, h, w, L.ax, L.ay, om, kEps, pl->gs, st));
            }
        }
        if (pl->store_sweeps)
            DCUDA(cudaMemcpyAsync(L.ck_final, s, (size_t)F * 2 * hw * sizeof(T), cudaMemcpyDeviceToDevice, st));
        DLAUNCH(1, median_add<T>(s, uv, (T*)pl->uvc[cur ^ 1], F, h, w, std::min(h, w) > 5 ? 1 : 0, st));
        cur ^= 1;
        prev = &L;
    }
    DCUDA(cudaMemcpyAsync(flow_out, pl->uvc[cur], (size_t)F * 2 * H * W * sizeof(T), cudaMemcpyDeviceToDevice, st));
    return FRG_OK;
}

template <typename T>
int run_backward(frg_diff_plan* pl, const T* g_flow, T* g_fixed, T* g_moving, double* g_alpha, int lagged,
                 int implicit, int stepwise, cudaStream_t st)
{
    using namespace frg::diff;
    const int F = pl->last_F, K = pl->K, H = pl->H, W = pl->W;
    const int I = pl->p.iterations, lag = pl->p.update_lag;
    const double om = pl->p.omega;
    const size_t es = sizeof(T);
    T* tmp = (T*)pl->tmp;
    if (g_fixed) DCUDA(cudaMemsetAsync(g_fixed, 0, (size_t)F * K * H * W * es, st));
    if (g_moving) DCUDA(cudaMemsetAsync(g_moving, 0, (size_t)F * K * H * W * es, st));
    double* galpha = g_alpha ? g_alpha : (double*)pl->galpha;
    DCUDA(cudaMemsetAsync(galpha, 0, (size_t)F * 2 * sizeof(double), st));
    const int W2 = (W + 1) / 2;
    DCUDA(cudaMemsetAsync(pl->partA, 0, (size_t)F * H * ((W2 + 127) / 128) * 2 * sizeof(double), st));
    DCUDA(cudaMemsetAsync(pl->partB, 0, (size_t)F * H * ((W + 127) / 128) * 2 * sizeof(double), st));
    DCUDA(cudaMemsetAsync(pl->partC, 0, (size_t)F * ((H + 15) / 16) * ((W + 15) / 16) * 2 * sizeof(double), st));
    int go = 0;
    DCUDA(cudaMemcpyAsync(pl->gout[go], g_flow, (size_t)F * 2 * H * W * es, cudaMemcpyDeviceToDevice, st));
    for (int li = (int)pl->levels.size() - 1; li >= 0; --li) {
        const DLevel& L = pl->levels[li];
        const int h = L.h, w = L.w;
        const long long hw = (long long)h * w;
        const size_t plane2 = (size_t)F * 2 * hw;
        const size_t slot = (size_t)F * 2 * h * ((w + 1) / 2);
        const double sx = L.scale / (L.h_col * L.h_col), sy = L.scale / (L.h_row * L.h_row);
        const T* f1 = (const T*)L.ck_f1;
        const T* f2 = (const T*)L.ck_f2;
        const T* uv = (const T*)L.ck_uv;
        const T* Wl = (const T*)L.Wl;
        T* J = (T*)pl->J;
        T* coef = (T*)pl->coef;
        T* gout = (T*)pl->gout[go];
        const T* f2w = f2;
        if (!L.top) {
            DLAUNCH(1, warp<T>(f2, f1, uv, F, K, h, w, L.h_col, L.h_row, (T*)pl->f2w, st));
            f2w = (const T*)pl->f2w;
        }
        DLAUNCH(1, tensor<T>(f1, f2w, F, K, h, w, L.h_row, L.h_col, J, st));
        T* gJ = (T*)pl->gJ;
        T* guv = (T*)pl->guv;
        T* gcoef = (T*)pl->gcoef;
        DCUDA(cudaMemsetAsync(gJ, 0, (size_t)F * 6 * K * hw * es, st));
        // u_out = u_in + median(du): the level's input flow receives g_out directly
        DCUDA(cudaMemcpyAsync(guv, gout, plane2 * es, cudaMemcpyDeviceToDevice, st));
        int lam_i = 0;
        T* lam = (T*)pl->lam[0];
        T* s = (T*)pl->st;
        // tiled window adjoints (one launch per window) unless stepwise is asked for or a window does not fit
        const int tile = stepwise ? 0 : pl->adj_tile;
        if (implicit) {
            // psi of the last tick, the level's final state, then one SOR solve of M lam = g
            const int k = pl->n_ticks - 1, start = k * lag, n_it = I - start;
            const T* s0 = k > 0 ? (const T*)L.ck_ticks + (size_t)(k - 1) * plane2 : nullptr;
            DLAUNCH(1, tick<T>(J, Wl, s0, uv, F, K, h, w, pl->a_data, kEps, L.ax, L.ay, coef, (T*)nullptr, st));
            const T* fin = (const T*)L.ck_final;
            if (!pl->store_sweeps) {
                if (s0)
                    DCUDA(cudaMemcpyAsync(s, s0, plane2 * es, cudaMemcpyDeviceToDevice, st));
                else
                    DCUDA(cudaMemsetAsync(s, 0, plane2 * es, st));
                for (int j = 0; j < 2 * n_it; ++j)
                    DLAUNCH(1, rb_sweep<T>(j & 1, coef, (const T*)nullptr, s, (T*)nullptr, F, h, w, L.ax, L.ay, om, kEps,
                                           pl->gs, st));
                fin = s;
            }
            T* g = (T*)pl->lam[1];
            if (std::min(h, w) > 5)
                DLAUNCH(2, median_adj<T>(fin, gout, pl->am, F, h, w, g, st));
            else
                DCUDA(cudaMemcpyAsync(g, gout, plane2 * es, cudaMemcpyDeviceToDevice, st));
            DCUDA(cudaMemsetAsync(lam, 0, plane2 * es, st));
            for (int it = 0; it < I; ++it)
                for (int c = 0; c < 2; ++c)
                    DLAUNCH(1, rb_sweep<T>(c, coef, g, lam, (T*)nullptr, F, h, w, L.ax, L.ay, om, kEps, 1, st));
            DLAUNCH(1, implicit_assemble<T>(lam, fin, F, h, w, gcoef, sx, sy, pl->partB, st));
            DLAUNCH(1, tick_adj<T>(J, Wl, s0, uv, gcoef, F, K, h, w, pl->a_data, kEps, L.ax, L.ay, 1, gJ, (T*)nullptr,
                                   guv, sx, sy, pl->partB, st));
        }
        for (int k = implicit ? -1 : pl->n_ticks - 1; k >= 0; --k) {
            const int start = k * lag, n_it = std::min(lag, I - start), n_half = 2 * n_it;
            const T* s0 = k > 0 ? (const T*)L.ck_ticks + (size_t)(k - 1) * plane2 : nullptr;
            if (pl->store_sweeps)
                coef = (T*)L.ck_coef + (size_t)k * F * 5 * hw;  // kept by the forward
            else
                DLAUNCH(1, tick<T>(J, Wl, s0, uv, F, K, h, w, pl->a_data, kEps, L.ax, L.ay, coef, (T*)nullptr, st));
            // the moved pixels of half-sweep j of this window
            T* base;
            if (pl->store_sweeps) {
                base = (T*)L.ck_sweeps + (size_t)(2 * start) * slot;
            } else {
                base = (T*)pl->states;
                if (s0)
                    DCUDA(cudaMemcpyAsync(s, s0, plane2 * es, cudaMemcpyDeviceToDevice, st));
                else
                    DCUDA(cudaMemsetAsync(s, 0, plane2 * es, st));
                for (int j = 0; j < n_half; ++j)
                    DLAUNCH(1, rb_sweep<T>(j & 1, coef, (const T*)nullptr, s, base + (size_t)j * slot, F, h, w, L.ax,
                                           L.ay, om, kEps, pl->gs, st));
            }
            if (k == pl->n_ticks - 1) {
                const T* fin = pl->store_sweeps ? (const T*)L.ck_final : s;
                if (std::min(h, w) > 5)
                    DLAUNCH(2, median_adj<T>(fin, gout, pl->am, F, h, w, lam, st));
                else
                    DCUDA(cudaMemcpyAsync(lam, gout, plane2 * es, cudaMemcpyDeviceToDevice, st));
            }
            if (tile) {
                // the window's half-sweeps in one tiled launch, lam into the other buffer
                T* lam_next = (T*)pl->lam[lam_i ^ 1];
                const AdjTable& tb = n_half == pl->adj_nh[0] ? pl->adj_tab[0] : pl->adj_tab[1];
                if (n_half != pl->adj_nh[0] && n_half != pl->adj_nh[1])
                    return host_fail(FRG_EINVAL, "no ring table for this window");
                DLAUNCH(1, rb_adj_window<T>(coef, s0, base, (long long)slot, lam, lam_next, F, h, w, n_half, tile, tb,
                                            L.ax, L.ay, om, kEps, pl->gs, gcoef, sx, sy, pl->partC, st));
                lam_i ^= 1;
                lam = lam_next;
            } else {
                DCUDA(cudaMemsetAsync(gcoef, 0, (size_t)F * 5 * hw * es, st));
                T* abuf[2] = {(T*)pl->abuf[0], (T*)pl->abuf[1]};
                const T* aprev = nullptr;
                for (int j = n_half - 1; j >= 0; --j) {
                    // before half-sweep j: its own colour last moved at j - 2, the other at j - 1
                    const T* own = j >= 2 ? base + (size_t)(j - 2) * slot : nullptr;
                    const T* oth = j >= 1 ? base + (size_t)(j - 1) * slot : nullptr;
                    const int c = j & 1;
                    const T* c0 = c == 0 ? own : oth;
                    const T* c1 = c == 0 ? oth : own;
                    T* anext = abuf[j & 1];
                    DLAUNCH(1, rb_adj_step<T>(c, coef, s0, c0, c1, lam, aprev, anext, F, h, w, L.ax, L.ay, om, kEps,
                                              pl->gs, gcoef, sx, sy, pl->partA, st));
                    aprev = anext;
                }
                DLAUNCH(1, rb_adj_gather<T>(1, lam, aprev, F, h, w, L.ax, L.ay, st));
            }
            DLAUNCH(1, tick_adj<T>(J, Wl, s0, uv, gcoef, F, K, h, w, pl->a_data, kEps, L.ax, L.ay, lagged, gJ,
                                   s0 ? lam : (T*)nullptr, guv, sx, sy, pl->partB, st));
        }
        DLAUNCH(1, reduce_slots(pl->partA, F, (long long)h * (((w + 1) / 2 + 127) / 128), galpha, st));
        if (tile && !implicit)
            DLAUNCH(1, reduce_slots(pl->partC, F, (long long)((h + tile - 1) / tile) * ((w + tile - 1) / tile), galpha,
                                    st));
        DLAUNCH(1, reduce_slots(pl->partB, F, (long long)h * ((w + 127) / 128), galpha, st));
        T* gf1 = (T*)pl->gf1;
        T* gf2w = (T*)pl->gf2w;
        DLAUNCH(2, tensor_adj<T>(f1, f2w, gJ, F, K, h, w, L.h_row, L.h_col, (T*)pl->G, gf1, gf2w, 0, st));
        T* gf2 = gf2w;
        if (!L.top) {
            gf2 = (T*)pl->gf2l;
            DCUDA(cudaMemsetAsync(gf2, 0, (size_t)F * K * hw * es, st));
            DLAUNCH(1, warp_adj<T>(f2, uv, gf2w, F, K, h, w, L.h_col, L.h_row, gf2, gf1, guv, st));
        }
        if (g_fixed)
            DLAUNCH(2, resize_t<T>(gf1, (long long)F * K, h, w, H, W, csr_x(L.img), csr_y(L.img), tmp, g_fixed, 1, st));
        if (g_moving)
            DLAUNCH(2, resize_t<T>(gf2, (long long)F * K, h, w, H, W, csr_x(L.img), csr_y(L.img), tmp, g_moving, 1,
                                   st));
        if (!L.top) {
            T* gnext = (T*)pl->gout[go ^ 1];
            DLAUNCH(2, resize_t<T>(guv, (long long)F * 2, h, w, L.sh, L.sw, csr_x(L.flow), csr_y(L.flow), tmp, gnext,
                                   0, st));
            go ^= 1;
        }
    }
    return FRG_OK;
}

}  // namespace

extern "C" {

int frg_diff_plan_create(const frg_params* params, int height, int width, int channels, int max_frames, int flags,
                         frg_diff_plan** out)
{
    if (!out || !params) return host_fail(FRG_EINVAL, "NULL argument");
    if (flags & ~(FRG_DIFF_TORCH_ORDER | FRG_DIFF_STORE_SWEEPS)) return host_fail(FRG_EINVAL, "unknown flags");
    *out = nullptr;
    if (height < 8 || width < 8) return host_fail(FRG_EINVAL, "frame must be at least 8 x 8");
    if (channels < 1 || channels > kMaxK) return host_fail(FRG_EINVAL, "channels must be in [1, 8]");
    if (max_frames < 1 || (long long)max_frames * std::max(channels, 2) > 65535)
        return host_fail(FRG_EINVAL, "max_frames out of range");
    if (params->iterations < 1 || params->update_lag < 1) return host_fail(FRG_EINVAL, "iterations/update_lag < 1");
    if (!(params->eta > 0.0 && params->eta <= 1.0)) return host_fail(FRG_EINVAL, "eta must be in (0, 1]");
    if (params->a_smooth != 1.0)
        return host_fail(FRG_EUNSUPPORTED, "the differentiable mode supports a_smooth = 1 only");
    if (params->const_assumption != 0)
        return host_fail(FRG_EUNSUPPORTED, "the differentiable mode supports gradient constancy only");
    if (params->gnc_stages != 0)
        return host_fail(FRG_EUNSUPPORTED, "the differentiable mode has no GNC stages");
    if (params->precision != FRG_FP32 && params->precision != FRG_FP64_REFERENCE)
        return host_fail(FRG_EINVAL, "precision must be FRG_FP32 or FRG_FP64_REFERENCE");

    // schedule: core/optical_flow.py:494-518
    const int m = height, n = width;
    const double eta = params->eta;
    int mly = host_warping_depth(eta, params->levels, m, m);
    int mlx = host_warping_depth(eta, params->levels, n, n);
    const int max_level = std::min(mlx, mly) * 4;
    mly = std::min(mly, max_level);
    mlx = std::min(mlx, max_level);
    const int top = std::max(mlx, mly);
    int min_level = params->min_level;
    if (top <= min_level) min_level = top - 1;
    if (min_level < 0) min_level = 0;
    if (min_level != 0)
        return host_fail(FRG_EUNSUPPORTED, "the differentiable mode computes down to level 0 (min_level 0)");

    frg_diff_plan* pl = new frg_diff_plan();
    pl->p = *params;
    pl->H = height;
    pl->W = width;
    pl->K = channels;
    pl->maxF = max_frames;
    pl->dbl = params->precision == FRG_FP64_REFERENCE;
    pl->es = pl->dbl ? 8 : 4;
    pl->alpha_x = params->alpha_x;
    pl->alpha_y = params->alpha_y;
    pl->gs = (flags & FRG_DIFF_TORCH_ORDER) ? 0 : 1;
    pl->store_sweeps = (flags & FRG_DIFF_STORE_SWEEPS) != 0;
    for (int k = 0; k < channels; ++k) pl->a_data[k] = params->a_data[k];
    const int I = params->iterations, lag = params->update_lag;
    pl->n_ticks = (I + lag - 1) / lag;
    pl->win = std::min(lag, I);
    const size_t F = (size_t)max_frames, K = (size_t)channels, es = pl->es;
    int rc = FRG_OK;
    int ph = 0, pw = 0;
    for (int i = top; i >= min_level && rc == FRG_OK; --i) {
        DLevel L;
        L.i = i;
        L.h = (int)std::nearbyint(m * std::pow(eta, (double)std::min(i, mly)));
        L.w = (int)std::nearbyint(n * std::pow(eta, (double)std::min(i, mlx)));
        if (L.h < 1 || L.w < 1) {
            rc = host_fail(FRG_EINVAL, "degenerate pyramid level");
            break;
        }
        L.top = (i == top);
        L.h_row = (double)m / L.h;
        L.h_col = (double)n / L.w;
        L.scale = (i == min_level) ? 1.0 : std::pow(eta, -0.5 * i);
        L.sh = L.top ? m : ph;
        L.sw = L.top ? n : pw;
        const size_t hw = (size_t)L.h * L.w;
        if ((rc = make_dtab(pl, &L.img, m, n, L.h, L.w)) || (rc = make_dtab(pl, &L.flow, L.sh, L.sw, L.h, L.w)) ||
            (rc = dalloc(pl, &L.Wl, K * hw * es)) || (rc = dalloc(pl, &L.ck_f1, F * K * hw * es)) ||
            (rc = dalloc(pl, &L.ck_f2, F * K * hw * es)) || (rc = dalloc(pl, &L.ck_uv, F * 2 * hw * es)) ||
            (rc = dalloc(pl, &L.ck_ticks, (size_t)std::max(pl->n_ticks - 1, 0) * F * 2 * hw * es)))
            break;
        if (pl->store_sweeps &&
            ((rc = dalloc(pl, &L.ck_sweeps, (size_t)2 * I * F * 2 * L.h * ((L.w + 1) / 2) * es)) ||
             (rc = dalloc(pl, &L.ck_final, F * 2 * hw * es)) ||
             (rc = dalloc(pl, &L.ck_coef, (size_t)pl->n_ticks * F * 5 * hw * es))))
            break;
        ph = L.h;
        pw = L.w;
        pl->levels.push_back(L);
    }
    const size_t hw = (size_t)height * width;  // the finest level is the largest
    if (rc == FRG_OK &&
        ((rc = dalloc(pl, &pl->tmp, F * std::max<size_t>(K, 2) * hw * es)) ||
         (rc = dalloc(pl, &pl->f2w, F * K * hw * es)) || (rc = dalloc(pl, &pl->J, F * 6 * K * hw * es)) ||
         (rc = dalloc(pl, &pl->coef, F * 5 * hw * es)) || (rc = dalloc(pl, &pl->st, F * 2 * hw * es)) ||
         (rc = dalloc(pl, &pl->uvc[0], F * 2 * hw * es)) || (rc = dalloc(pl, &pl->uvc[1], F * 2 * hw * es)) ||
         (rc = dalloc(pl, &pl->states, pl->store_sweeps ? 16 : (size_t)(2 * pl->win) * F * 2 * height *
                                                                      ((width + 1) / 2) * es)) ||
         (rc = dalloc(pl, &pl->lam[0], F * 2 * hw * es)) || (rc = dalloc(pl, &pl->lam[1], F * 2 * hw * es)) ||
         (rc = dalloc(pl, &pl->abuf[0], F * 2 * height * ((width + 1) / 2) * es)) ||
         (rc = dalloc(pl, &pl->abuf[1], F * 2 * height * ((width + 1) / 2) * es)) ||
         (rc = dalloc(pl, &pl->gcoef, F * 5 * hw * es)) || (rc = dalloc(pl, &pl->guv, F * 2 * hw * es)) ||
         (rc = dalloc(pl, &pl->galpha, F * 2 * sizeof(double))) ||
         (rc = dalloc_t(pl, &pl->partA, F * height * (size_t)(((width + 1) / 2 + 127) / 128) * 2)) ||
         (rc = dalloc_t(pl, &pl->partB, F * height * (size_t)((width + 127) / 128) * 2)) ||
         (rc = dalloc_t(pl, &pl->partC, F * (size_t)((height + 15) / 16) * ((width + 15) / 16) * 2)) || (rc = dalloc(pl, &pl->gJ, F * 6 * K * hw * es)) ||
         (rc = dalloc(pl, &pl->G, F * 5 * K * hw * es)) || (rc = dalloc(pl, &pl->gf1, F * K * hw * es)) ||
         (rc = dalloc(pl, &pl->gf2w, F * K * hw * es)) || (rc = dalloc(pl, &pl->gf2l, F * K * hw * es)) ||
         (rc = dalloc(pl, &pl->gout[0], F * 2 * hw * es)) || (rc = dalloc(pl, &pl->gout[1], F * 2 * hw * es)) ||
         (rc = dalloc_t(pl, &pl->am, F * 2 * hw))))
        ;
    if (rc == FRG_OK) rc = make_adj_tables(pl);
    if (rc != FRG_OK) {
        frg_diff_plan_destroy(pl);
        return rc;
    }
    *out = pl;
    return FRG_OK;
}

void frg_diff_plan_destroy(frg_diff_plan* plan)
{
    if (!plan) return;
    cudaDeviceSynchronize();
    for (void* p : plan->allocs) cudaFree(p);
    delete plan;
}

size_t frg_diff_plan_device_bytes(const frg_diff_plan* plan) { return plan ? plan->bytes : 0; }

int frg_diff_plan_num_levels(const frg_diff_plan* plan) { return plan ? (int)plan->levels.size() : 0; }

int frg_diff_set_level_tables(frg_diff_plan* plan, int level, int kind, int taps, const int* ix, const float* wx,
                              const int* iy, const float* wy)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return host_fail(FRG_EINVAL, "bad level");
    if (kind != 0 && kind != 1) return host_fail(FRG_EINVAL, "kind must be 0 (image) or 1 (flow)");
    if (!ix || !wx || !iy || !wy) return host_fail(FRG_EINVAL, "NULL table");
    DTab& d = kind == 0 ? plan->levels[level].img : plan->levels[level].flow;
    if (taps != d.P) return host_fail(FRG_EINVAL, "tap count differs from the plan's");
    for (size_t i = 0; i < (size_t)d.out_w * taps; ++i)
        if (ix[i] < 0 || ix[i] >= d.in_w) return host_fail(FRG_EINVAL, "column index out of range");
    for (size_t i = 0; i < (size_t)d.out_h * taps; ++i)
        if (iy[i] < 0 || iy[i] >= d.in_h) return host_fail(FRG_EINVAL, "row index out of range");
    return put_tables(plan, &d, ix, wx, iy, wy);
}

int frg_diff_set_weight(frg_diff_plan* pl, const void* weight, void* stream)
{
    if (!pl || !weight) return host_fail(FRG_EINVAL, "plan or weight is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    for (DLevel& L : pl->levels) {
        if (pl->dbl)
            DLAUNCH(2, diff::resize<double>((const double*)weight, pl->K, pl->H, pl->W, L.h, L.w, L.img.ix, L.img.wx,
                                            L.img.P, L.img.iy, L.img.wy, L.img.P, (double*)pl->tmp, (double*)L.Wl, st));
        else
            DLAUNCH(2, diff::resize<float>((const float*)weight, pl->K, pl->H, pl->W, L.h, L.w, L.img.ix, L.img.wx,
                                           L.img.P, L.img.iy, L.img.wy, L.img.P, (float*)pl->tmp, (float*)L.Wl, st));
    }
    pl->has_weight = true;
    return FRG_OK;
}

int frg_diff_forward(frg_diff_plan* pl, int n_frames, double alpha_x, double alpha_y, const void* fixed,
                     const void* moving, const void* uv_init, void* flow_out, void* stream)
{
    if (!pl || !fixed || !moving || !flow_out) return host_fail(FRG_EINVAL, "NULL argument");
    if (n_frames < 1 || n_frames > pl->maxF) return host_fail(FRG_EINVAL, "n_frames out of range");
    if (!pl->has_weight) return host_fail(FRG_EINVAL, "frg_diff_set_weight was not called");
    pl->alpha_x = alpha_x;
    pl->alpha_y = alpha_y;
    pl->last_F = n_frames;
    pl->have_forward = false;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = pl->dbl ? run_forward<double>(pl, n_frames, (const double*)fixed, (const double*)moving,
                                           (const double*)uv_init, (double*)flow_out, st)
                     : run_forward<float>(pl, n_frames, (const float*)fixed, (const float*)moving,
                                          (const float*)uv_init, (float*)flow_out, st);
    if (rc == FRG_OK) pl->have_forward = true;
    return rc;
}

int frg_diff_backward(frg_diff_plan* pl, const void* g_flow, void* g_fixed, void* g_moving, double* g_alpha,
                      int flags, void* stream)
{
    if (!pl || !g_flow) return host_fail(FRG_EINVAL, "NULL argument");
    if (flags & ~(FRG_DIFF_LAGGED_PSI | FRG_DIFF_IMPLICIT | FRG_DIFF_STEPWISE_ADJOINT))
        return host_fail(FRG_EINVAL, "unknown flags");
    if (!pl->have_forward) return host_fail(FRG_EINVAL, "no forward pass to differentiate");
    cudaStream_t st = (cudaStream_t)stream;
    const int lagged = (flags & FRG_DIFF_LAGGED_PSI) ? 1 : 0, implicit = (flags & FRG_DIFF_IMPLICIT) ? 1 : 0;
    const int stepwise = (flags & FRG_DIFF_STEPWISE_ADJOINT) ? 1 : 0;
    return pl->dbl ? run_backward<double>(pl, (const double*)g_flow, (double*)g_fixed, (double*)g_moving, g_alpha,
                                          lagged, implicit, stepwise, st)
                   : run_backward<float>(pl, (const float*)g_flow, (float*)g_fixed, (float*)g_moving, g_alpha, lagged,
                                         implicit, stepwise, st);
}

int frg_diff_warp(int precision, int n_frames, int channels, int height, int width, const void* src,
                  const void* flow, const void* fill, void* out, void* stream)
{
    if (!src || !flow || !fill || !out) return host_fail(FRG_EINVAL, "NULL argument");
    if (n_frames < 1 || n_frames > 65535 || channels < 1 || height < 1 || width < 1)
        return host_fail(FRG_EINVAL, "bad shape");
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == FRG_FP64_REFERENCE)
        DLAUNCH(1, diff::warp<double>((const double*)src, (const double*)fill, (const double*)flow, n_frames, channels,
                                      height, width, 1.0, 1.0, (double*)out, st));
    else if (precision == FRG_FP32)
        DLAUNCH(1, diff::warp<float>((const float*)src, (const float*)fill, (const float*)flow, n_frames, channels,
                                     height, width, 1.0, 1.0, (float*)out, st));
    else
        return host_fail(FRG_EINVAL, "precision must be FRG_FP32 or FRG_FP64_REFERENCE");
    return FRG_OK;
}

int frg_diff_warp_backward(int precision, int n_frames, int channels, int height, int width, const void* src,
                           const void* flow, const void* g_out, void* g_src, void* g_fill, void* g_flow,
                           void* stream)
{
    if (!src || !flow || !g_out || !g_src) return host_fail(FRG_EINVAL, "NULL argument");
    if (n_frames < 1 || n_frames > 65535 || channels < 1 || height < 1 || width < 1)
        return host_fail(FRG_EINVAL, "bad shape");
    if (precision != FRG_FP32 && precision != FRG_FP64_REFERENCE)
        return host_fail(FRG_EINVAL, "precision must be FRG_FP32 or FRG_FP64_REFERENCE");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t es = precision == FRG_FP64_REFERENCE ? 8 : 4;
    const size_t img = (size_t)n_frames * channels * height * width * es;
    DCUDA(cudaMemsetAsync(g_src, 0, img, st));
    if (g_fill) DCUDA(cudaMemsetAsync(g_fill, 0, img, st));
    if (g_flow) DCUDA(cudaMemsetAsync(g_flow, 0, (size_t)n_frames * 2 * height * width * es, st));
    if (precision == FRG_FP64_REFERENCE)
        DLAUNCH(1, diff::warp_adj<double>((const double*)src, (const double*)flow, (const double*)g_out, n_frames,
                                          channels, height, width, 1.0, 1.0, (double*)g_src, (double*)g_fill,
                                          (double*)g_flow, st));
    else
        DLAUNCH(1, diff::warp_adj<float>((const float*)src, (const float*)flow, (const float*)g_out, n_frames, channels,
                                         height, width, 1.0, 1.0, (float*)g_src, (float*)g_fill, (float*)g_flow, st));
    return FRG_OK;
}

}  // extern "C"
