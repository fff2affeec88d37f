// C ABI and host orchestration of the GB300 optical-flow path.
//
// The plan mirrors the level loop of pyflowreg's _solve_displacement_stage
// (src/pyflowreg/core/optical_flow.py:476-617): the pyramid schedule
// (warpingDepth, core/warping.py:237-277), the resize tap tables
// (util/resize_util.py:182-229) and the alpha scaling are computed on the host
// once per plan; every level then runs a fixed sequence of kernels over the
// whole batch of frames.
#include "frg_internal.h"
#include "../../include/flowreg_gb300.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <vector>

using namespace frg;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

#define FRG_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(FRG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
    } while (0)

// Every kernel launch made by this library goes through FRG_LAUNCH, which
// counts it (frg_launch_count) so a caller can state how many kernels ran.
std::atomic<long long> g_launches{0};
#define FRG_LAUNCH(call)                                                                    \
    do {                                                                                    \
        g_launches.fetch_add(1, std::memory_order_relaxed);                                 \
        FRG_CUDA(call);                                                                     \
    } while (0)

// ---------------------------------------------------------------------------
// Host-side schedule and tables.
// ---------------------------------------------------------------------------

// warpingDepth (core/warping.py:237-277); Python round() is round-half-even.
int warping_depth(double eta, int levels, int m, int n)
{
    double min_dim = std::min(m, n);
    int depth = 0;
    for (int i = 0; i < levels; ++i) {
        ++depth;
        min_dim *= eta;
        if (std::nearbyint(min_dim) < 10) break;
    }
    return depth;
}

// Keys cubic with A = -0.75 (util/resize_util.py:68-76), double precision.
double keys(double x)
{
    const double A = -0.75;
    const double ax = std::fabs(x);
    if (ax < 1.0) return (A + 2.0) * std::pow(ax, 3.0) - (A + 3.0) * ax * ax + 1.0;
    if (ax < 2.0) return A * std::pow(ax, 3.0) - 5.0 * A * ax * ax + 8.0 * A * ax - 4.0 * A;
    return 0.0;
}

int reflect_idx(int j, int n)
{
    if (n <= 1) return 0;
    while (j < 0 || j >= n) j = j < 0 ? -j - 1 : 2 * n - 1 - j;
    return j;
}

// numpy's float32 sum of a small contiguous array (add.reduce: first element,
// then the pairwise block of the rest with eight partial sums).
float np_sum_f32(const std::vector<float>& a)
{
    if (a.empty()) return 0.0f;
    const float* p = a.data() + 1;
    const long n = (long)a.size() - 1;
    float rest = 0.0f;
    if (n < 8) {
        for (long i = 0; i < n; ++i) rest += p[i];
    } else {
        float r[8];
        for (int j = 0; j < 8; ++j) r[j] = p[j];
        long i = 8;
        for (; i < n - (n % 8); i += 8)
            for (int j = 0; j < 8; ++j) r[j] += p[i + j];
        rest = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; ++i) rest += p[i];
    }
    return a[0] + rest;
}

struct HostTables {
    int P = 0;
    std::vector<int32_t> idx;
    std::vector<float> wt;
};

// _precompute_fused_gauss_cubic + _fill_tables_fused_gauss_cubic_reflect
// (util/resize_util.py:194-229) with numba's typing: float32 Gaussian taps,
// float64 accumulation and normalisation, float32 stores.
HostTables make_tables(int in_len, int out_len, double sigma)
{
    HostTables t;
    const double scale = (double)out_len / (double)in_len;
    int R = 0;
    std::vector<float> g;
    if (sigma <= 0.0) {
        g.push_back(1.0f);
    } else {
        R = (int)std::ceil(2.0 * sigma);
        const float sf = (float)sigma;
        for (int u = -R; u <= R; ++u) {
            volatile float q = (float)u / sf;
            volatile float q2 = q * q;
            volatile float e = -0.5f * q2;
            g.push_back(std::exp(e));
        }
        const float s = np_sum_f32(g);
        for (float& x : g) x = x / s;
    }
    t.P = 2 * R + 4;
    t.idx.resize((size_t)out_len * t.P);
    t.wt.resize((size_t)out_len * t.P);
    std::vector<double> acc(t.P);
    for (int i = 0; i < out_len; ++i) {
        const double x = (i + 0.5) / scale - 0.5;
        const int left = (int)std::floor(x - 2.0) - R;
        double ssum = 0.0;
        for (int p = 0; p < t.P; ++p) {
            const int j = left + p;
            t.idx[(size_t)i * t.P + p] = reflect_idx(j, in_len);
            const double d = x - j;
            double a = 0.0;
            for (int u = -R; u <= R; ++u) a += (double)g[u + R] * keys(d - u);
            t.wt[(size_t)i * t.P + p] = (float)a;
            ssum += a;
        }
        const double inv = 1.0 / ssum;
        for (int p = 0; p < t.P; ++p)
            t.wt[(size_t)i * t.P + p] = (float)((double)t.wt[(size_t)i * t.P + p] * inv);
    }
    return t;
}

// sigma of imresize_fused_gauss_cubic (util/resize_util.py:235-242)
double resize_sigma(int ih, int iw, int oh, int ow)
{
    const double sy = (double)oh / ih, sx = (double)ow / iw;
    const double s = sy < sx ? sy : sx;
    return s < 1.0 ? 0.6 / s : 0.0;
}

// The four Keys (A = -0.75) weights OpenCV documents for bicubic sampling at
// fractional offset t (taps at distances 1+t, t, 1-t, 2-t; the last is one
// minus the others), single precision with a fixed operation order.
void keys4(float tf, float* out)
{
    volatile float t = tf;
    const float A = -0.75f;
    auto inner = [&](float x) {
        volatile float a = (A + 2.0f) * x;
        volatile float b = a - (A + 3.0f);
        volatile float xx = x * x;
        volatile float c = b * xx;
        return (float)(c + 1.0f);
    };
    auto outer = [&](float x) {
        volatile float a = A * x;
        volatile float b = a - 5.0f * A;
        volatile float c = b * x;
        volatile float d = c + 8.0f * A;
        volatile float e = d * x;
        return (float)(e - 4.0f * A);
    };
    const float w0 = outer(1.0f + t);
    const float w1 = inner(t);
    const float w2 = inner(1.0f - t);
    volatile float r = 1.0f - w0;
    r = r - w1;
    r = r - w2;
    out[0] = w0;
    out[1] = w1;
    out[2] = w2;
    out[3] = r;
}

// cv2.remap weights at the 32 sub-pixel positions (bicubic and bilinear).
void remap_tables(float* cub, float* lin)
{
    for (int k = 0; k < 32; ++k) {
        volatile float t = (float)k / 32.0f;
        keys4(t, cub + k * 4);
        lin[k * 2 + 0] = 1.0f - t;
        lin[k * 2 + 1] = t;
    }
}

// Tap start and weights of cv2.resize INTER_CUBIC along one axis
// (in_len -> out_len): source coordinate (d + 0.5) * in/out - 0.5.
void upsample_tables(int in_len, int out_len, std::vector<int32_t>& s0, std::vector<float>& wt)
{
    s0.resize(out_len);
    wt.resize((size_t)out_len * 4);
    const double scale = (double)in_len / (double)out_len;
    for (int d = 0; d < out_len; ++d) {
        const double f = (d + 0.5) * scale - 0.5;
        const double s = std::floor(f);
        s0[d] = (int32_t)s;
        keys4((float)(f - s), wt.data() + (size_t)d * 4);
    }
}

// The tables live in __constant__ memory, which every device holds separately:
// uploaded once per device, under a lock (plans may be created from several
// threads).
int ensure_remap_tables()
{
    static std::mutex mu;
    static std::set<int> done;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(FRG_ECUDA, "no CUDA device");
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(dev)) return FRG_OK;
    float cub[128], lin[64];
    remap_tables(cub, lin);
    FRG_CUDA(upload_cubic_table(cub, lin));
    FRG_CUDA(upload_cubic_table_x(cub));
    FRG_CUDA(upload_dpow_tables());
    done.insert(dev);
    return FRG_OK;
}

DiagGeom make_geom(int h, int w)
{
    DiagGeom g;
    g.h = h;
    g.w = w;
    g.D = h + w - 1;
    g.P = (h + 31) / 32 * 32;
    return g;
}

struct DevTables {
    int P = 0;
    int32_t* ix = nullptr;
    float* wx = nullptr;
    int32_t* iy = nullptr;
    float* wy = nullptr;
};

struct LevelPlan {
    int i = 0;         // pyramid index (coarsest = largest)
    int h = 0, w = 0;  // level size
    bool top = false;
    double h_row = 1, h_col = 1, alpha_x = 0, alpha_y = 0;
    float wx = 0, wy = 0;  // alpha_x / h_col^2, alpha_y / h_row^2
    DiagGeom g{};
    int fh = 0, fw = 0;   // flow source size (previous level; full size at the top)
    DevTables img, flow;  // full-res -> level, flow source -> level
    float* ref = nullptr;    // (K, h, w) reference level
    float* wdiag = nullptr;  // (K, D*P) weight level, diagonal-major
    double* wpad64 = nullptr;  // (K, (h+2)*(w+2)) weight level with zero ring (fp64 mode)
    double* wdiag64 = nullptr;  // (2, K, D*P) the same and times a_data, diagonal-major, for the float64 chained SOR
    double* ref64 = nullptr;    // (K, h, w) reference level in float64, for its tensor
    double* refd64 = nullptr;   // (4, K, h, w) its derivatives gx1, gy1, fxx1, fyy1 (launch_x_ref_derivs)
    bool chain64 = false;       // fp64 plan: this level runs the float64 chained SOR
    int rows64 = 0;             // its rows per CTA strip (64, 128, 256); 0: chosen per call from the batch size
    int sor_G = 0;        // fused SOR iterations per pass (0: the most the ring allows)
    int sor_threads = 0;  // fused SOR threads per CTA (0: the level's rows, P)
    int sor_variant = 0;  // fused SOR kernel: 0 diagonal ring in shared memory, 1 rows with the state in registers
                          // (one launch per pass), 2 the same with every pass of the level in one launch (the
                          // default where it serves)
};

// Iteration groups between nonlinearity ticks ((t+1) % update_lag == 0,
// core/level_solver.py:230), split into wavefront passes of <= kGMax.
struct Pass {
    int G;
    int fold_mode;  // -1: no fold; else bit0 zero-init, bit1 psi from (du, dv)
};

// Writes the passes into out[0, cap) (out may be NULL) and returns how many
// there are; allocates nothing.
int fill_passes(int iterations, int update_lag, int gmax, Pass* out, int cap)
{
    int n = 0;
    int t = 0;
    while (t < iterations) {
        const bool tick = ((t + 1) % update_lag) == 0;
        int end = t + 1;
        while (end < iterations && ((end + 1) % update_lag) != 0) ++end;
        int mode = (t == 0 ? 1 : 0) | (tick ? 2 : 0);
        for (int s = t; s < end; s += gmax) {
            if (out && n < cap) {
                out[n].G = std::min(gmax, end - s);
                out[n].fold_mode = (s == t) ? mode : -1;
            }
            ++n;
        }
        t = end;
    }
    return n;
}

std::vector<Pass> make_passes(int iterations, int update_lag, int gmax = kGMax)
{
    std::vector<Pass> out((size_t)fill_passes(iterations, update_lag, gmax, nullptr, 0));
    fill_passes(iterations, update_lag, gmax, out.data(), (int)out.size());
    return out;
}

// Chain table of a level's passes (every pass in one k_sor_chain launch): a
// group's first pass stores its folded coefficients when the group continues
// in further passes, which read them back.  Returns the iterations summed.
int chain_passes(const Pass* ps, int n, ChainPass* cp)
{
    int its = 0;
    for (int pi = 0; pi < n; ++pi) {
        const bool continued = pi + 1 < n && ps[pi + 1].fold_mode < 0;
        cp[pi].G = ps[pi].G;
        cp[pi].mode = ps[pi].fold_mode;
        cp[pi].store_coef = (ps[pi].fold_mode >= 0 && continued) ? 1 : 0;
        its += ps[pi].G;
    }
    return its;
}

// CUDA-event timing of every SOR launch, enabled by frg_plan_set_profiling.
// Algorithmic bytes of one launch: per interior pixel and pipelined
// iteration, five coefficients and du, dv read plus du, dv written (36 B).
struct SorProfile {
    bool on = false;
    std::vector<cudaEvent_t> ev;  // begin/end pairs
    size_t used = 0;
    double bytes = 0.0;
    long long launches = 0;
};

}  // namespace

struct frg_plan {
    frg_params p{};
    frg_level_solver_fn solver_fn = nullptr;  // host level solver in place of the float64 SOR
    void* solver_user = nullptr;
    int H = 0, W = 0, K = 0, max_T = 0;
    int min_level = 0;
    std::vector<LevelPlan> levels;
    std::vector<void*> allocs;
    size_t bytes = 0;
    bool has_ref = false;
    // per-batch workspace
    float* tmp = nullptr;     // horizontal resize pass
    float* f2 = nullptr;      // (T, K, h, w)
    float* warped = nullptr;  // (T, K, h, w)
    float* J = nullptr;       // (T, 6, K, D*P)
    float* lap = nullptr;     // (T, 2, D*P)
    float* coef = nullptr;    // (T, 5, D*P)
    float* du = nullptr;      // (T, D*P)
    float* dv = nullptr;      // (T, D*P)
    float* uvpad = nullptr;   // (T, 2, h+2, w+2)
    float* uacc[2] = {nullptr, nullptr};  // (T, 2, h, w)
    float* durm = nullptr;    // (2, T, h, w): the level's final du, dv, row-major
    float* ones = nullptr;    // (H, W, K) default weight
    float a_data[kMaxK] = {0};
    SorProfile prof;
    // FP64 reference-order workspace (precision == FRG_FP64_REFERENCE)
    double* xJ = nullptr;     // (T, 6, K, m*n)
    double* xwp = nullptr;    // (T, K, m*n) weight * psi
    double* xdu = nullptr;    // (T, m*n)
    double* xdv = nullptr;    // (T, m*n)
    double* xuv = nullptr;    // (T, 2, m*n)
    double* xacc[2] = {nullptr, nullptr};  // (T, 2, h*w)
    double a_data64[kMaxK] = {0};
    PowTab64 pow64[kMaxK];  // the float64 chained SOR's power table per channel (shared by equal exponents)
    // final cubic upsampling when min_level > 0 (tables per output column / row)
    int32_t* up_sx = nullptr;
    float* up_wx = nullptr;
    int32_t* up_sy = nullptr;
    float* up_wy = nullptr;
    double* xtmp = nullptr;   // fp64 width-pass buffer (T, 2, h_min, W)
    // a_smooth != 1, the census data term and GNC stages run on the reference-order kernels in both precisions
    bool xpath = false;       // precision == FRG_FP64_REFERENCE, a_smooth != 1, census or GNC
    // FP64 plans with a_smooth = 1, gradient or gray-value constancy and no GNC: the
    // levels the float64 chained SOR serves run it on diagonal-major float64 buffers
    bool dpath = false;
    int n_sms = 0;            // multiprocessors of the plan's device
    double* dJ = nullptr;     // (T, 6, K, D*P)
    double* dlap = nullptr;   // (T, 2, D*P)
    double* dcoef = nullptr;  // (T, 5, D*P)
    double* ddu = nullptr;    // (T, D*P)
    double* ddv = nullptr;    // (T, D*P)
    double* xpsis = nullptr;  // (T, m*n) smoothness weights
    double* xsnap = nullptr;  // (T, 2, m*n) state snapshot for the psi_s border
    double* xflow = nullptr;  // (T, H, W, 2) fp64 flow of an fp32 plan on this path
};

namespace {

template <typename T>
int dev_alloc(frg_plan* pl, T** out, size_t count)
{
    void* p = nullptr;
    const size_t b = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) return fail(FRG_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    pl->allocs.push_back(p);
    pl->bytes += b;
    *out = (T*)p;
    return FRG_OK;
}

// The float64 chained SOR's power tables: one per distinct exponent a_data[k] - 1
// with |a_data[k] - 1| <= 1 (others keep a null table: the general power).
int make_pow_tables(frg_plan* pl, int channels)
{
    std::vector<double2> tab(kPowTabN);
    for (int k = 0; k < channels; ++k) {
        const double b = pl->a_data64[k] - 1.0;
        int same = -1;
        for (int q = 0; q < k && same < 0; ++q)
            if (pl->a_data64[q] - 1.0 == b) same = q;
        if (same >= 0) {
            pl->pow64[k] = pl->pow64[same];
            continue;
        }
        PowTab64 pt;
        if (!make_pow_table(b, tab.data(), &pt)) continue;
        double2* dt = nullptr;
        if (int rc = dev_alloc(pl, &dt, (size_t)kPowTabN)) return rc;
        const cudaError_t e = cudaMemcpy(dt, tab.data(), sizeof(double2) * kPowTabN, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(FRG_ECUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        pt.t = dt;
        pl->pow64[k] = pt;
    }
    return FRG_OK;
}

int upload_tables(frg_plan* pl, const HostTables& t, int n_out_x, const HostTables& ty, int n_out_y,
                  DevTables* d)
{
    (void)n_out_x;
    (void)n_out_y;
    d->P = t.P;
    int rc;
    if ((rc = dev_alloc(pl, &d->ix, t.idx.size()))) return rc;
    if ((rc = dev_alloc(pl, &d->wx, t.wt.size()))) return rc;
    if ((rc = dev_alloc(pl, &d->iy, ty.idx.size()))) return rc;
    if ((rc = dev_alloc(pl, &d->wy, ty.wt.size()))) return rc;
    FRG_CUDA(cudaMemcpy(d->ix, t.idx.data(), t.idx.size() * 4, cudaMemcpyHostToDevice));
    FRG_CUDA(cudaMemcpy(d->wx, t.wt.data(), t.wt.size() * 4, cudaMemcpyHostToDevice));
    FRG_CUDA(cudaMemcpy(d->iy, ty.idx.data(), ty.idx.size() * 4, cudaMemcpyHostToDevice));
    FRG_CUDA(cudaMemcpy(d->wy, ty.wt.data(), ty.wt.size() * 4, cudaMemcpyHostToDevice));
    return FRG_OK;
}

View view(const float* p, long long fs, long long ps, long long rs, long long cs)
{
    View v;
    v.p = p;
    v.fs = fs;
    v.ps = ps;
    v.rs = rs;
    v.cs = cs;
    return v;
}

ViewW vieww(float* p, long long fs, long long ps, long long rs, long long cs)
{
    ViewW v;
    v.p = p;
    v.fs = fs;
    v.ps = ps;
    v.rs = rs;
    v.cs = cs;
    return v;
}

int record_event(SorProfile* pr, cudaStream_t st)
{
    if (pr->used == pr->ev.size()) {
        cudaEvent_t e;
        FRG_CUDA(cudaEventCreate(&e));
        pr->ev.push_back(e);
    }
    FRG_CUDA(cudaEventRecord(pr->ev[pr->used++], st));
    return FRG_OK;
}

// Runs the passes of one level.  K <= 4: one fused launch per pass (the fold
// happens in the SOR's loader; a group cut into several passes stores its
// coefficients in its first pass and the others read them).  Larger K: a fold
// kernel at each group start, then the row-per-thread SOR.
// Which SOR kernel a level uses: the fused shared-memory ring (K <= 4, up to
// 1024 rows), the row-per-thread ring with a separate fold (K > 4, up to 512
// rows), or the global-memory wavefront with a separate fold (anything else).
enum SorKind { kSorFused = 0, kSorRows = 1, kSorGlobal = 2 };

SorKind sor_kind(int K, const DiagGeom& g)
{
    if (sor_fused_supports(K) && sor_fused_gmax(g.P) >= 1) return kSorFused;
    if (g.P <= kMaxLane) return kSorRows;
    return kSorGlobal;
}

int solve_level(int iterations, int update_lag, const float* J, long long J_fs, const float* W,
                long long W_fs, const float* lap, long long lap_fs, float* du, float* dv,
                long long st_fs, float* coef, long long coef_fs, int T, int K, const DiagGeom& g,
                const float* a_data, float wx, float wy, float omega, cudaStream_t st,
                SorProfile* prof = nullptr, float* rm_du = nullptr, float* rm_dv = nullptr, long long rm_fs = 0,
                int tune_G = 0, int tune_threads = 0, int tune_variant = 0)
{
    const SorKind kind = sor_kind(K, g);
    const bool regs = tune_variant >= 1 && sor_regs_supports(K, g);
    const bool fused = kind == kSorFused && !regs;
    int gmax = regs ? kGMax : (kind == kSorFused ? sor_fused_gmax(g.P) : (kind == kSorRows ? kGMax : update_lag));
    if ((fused || regs) && tune_G > 0 && tune_G < gmax) gmax = tune_G;
    const std::vector<Pass> passes = make_passes(iterations, update_lag, gmax);
    if (regs && tune_variant == 2 && sor_chain_supports(K, g, (int)passes.size())) {
        // every pass in one launch; same arguments per pass as the loop below
        std::vector<ChainPass> cp(passes.size());
        const double its = chain_passes(passes.data(), (int)passes.size(), cp.data());
        const bool timed = prof && prof->on;
        if (timed) {
            int rc = record_event(prof, st);
            if (rc) return rc;
        }
        FRG_LAUNCH(launch_sor_chain(J, J_fs, W, W_fs, lap, lap_fs, coef, coef_fs, du, dv, st_fs, T, K, g, cp.data(),
                                    (int)cp.size(), a_data, wx, wy, omega, st, rm_du, rm_dv, rm_fs));
        if (timed) {
            int rc = record_event(prof, st);
            if (rc) return rc;
            prof->bytes += 36.0 * its * (double)T * g.h * g.w;
            prof->launches += 1;
        }
        return FRG_OK;
    }
    for (size_t pi = 0; pi < passes.size(); ++pi) {
        const Pass& ps = passes[pi];
        if (!fused && !regs && ps.fold_mode >= 0)
            FRG_LAUNCH(launch_fold(J, J_fs, W, W_fs, lap, lap_fs, du, dv, st_fs, coef, coef_fs, T, K, g,
                                   a_data, ps.fold_mode, wx, wy, st));
        const bool timed = prof && prof->on;
        if (timed) {
            int rc = record_event(prof, st);
            if (rc) return rc;
        }
        if (regs) {
            const bool continued = pi + 1 < passes.size() && passes[pi + 1].fold_mode < 0;
            const bool final_pass = pi + 1 == passes.size();
            FRG_LAUNCH(launch_sor_regs(J, J_fs, W, W_fs, lap, lap_fs, coef, coef_fs, du, dv, st_fs, T, K, g, ps.G,
                                       ps.fold_mode, (ps.fold_mode >= 0 && continued) ? 1 : 0, a_data, wx, wy, omega,
                                       st, final_pass ? rm_du : nullptr, final_pass ? rm_dv : nullptr, rm_fs));
        } else if (fused) {
            const bool continued = pi + 1 < passes.size() && passes[pi + 1].fold_mode < 0;
            const bool final_pass = pi + 1 == passes.size();
            FRG_LAUNCH(launch_sor_fused(J, J_fs, W, W_fs, lap, lap_fs, coef, coef_fs, du, dv, st_fs, T, K, g, ps.G,
                                        ps.fold_mode, (ps.fold_mode >= 0 && continued) ? 1 : 0, a_data, wx, wy,
                                        omega, st, final_pass ? rm_du : nullptr, final_pass ? rm_dv : nullptr,
                                        rm_fs, tune_threads));
        } else if (kind == kSorRows) {
            // thread index runs along rows: rows are the a-direction (weight wy)
            FRG_LAUNCH(launch_sor(coef, coef_fs, du, dv, st_fs, T, g, ps.G, wy, wx, omega, st));
        } else {
            FRG_LAUNCH(launch_sor_global(coef, coef_fs, du, dv, st_fs, T, g, ps.G, wy, wx, omega, st));
        }
        if (timed) {
            int rc = record_event(prof, st);
            if (rc) return rc;
            prof->bytes += 36.0 * ps.G * (double)T * g.h * g.w;
            prof->launches += 1;
        }
    }
    return FRG_OK;
}

int check_params(const frg_params* p, int K)
{
    if (!p) return fail(FRG_EINVAL, "params is NULL");
    if (!(p->eta > 0.0 && p->eta <= 1.0)) return fail(FRG_EINVAL, "eta must be in (0, 1]");
    if (p->levels < 1) return fail(FRG_EINVAL, "levels must be >= 1");
    if (p->iterations < 1) return fail(FRG_EINVAL, "iterations must be >= 1");
    if (p->update_lag < 1) return fail(FRG_EINVAL, "update_lag must be >= 1");
    if (p->min_level < 0) return fail(FRG_EINVAL, "min_level must be >= 0");
    if (!(p->a_smooth > 0.0)) return fail(FRG_EINVAL, "a_smooth must be > 0");
    if (p->const_assumption < 0 || p->const_assumption > 2)
        return fail(FRG_EINVAL, "const_assumption must be 0 (gc), 1 (gray) or 2 (census)");
    for (int k = 0; k < K; ++k)
        if (!(p->a_data[k] > 0.0)) return fail(FRG_EINVAL, "a_data must be > 0");
    if (p->precision != FRG_FP32 && p->precision != FRG_FP64_REFERENCE)
        return fail(FRG_EINVAL, "precision must be FRG_FP32 or FRG_FP64_REFERENCE");
    if (p->gnc_stages != 0) {
        // normalize_gnc_schedule / normalize_warping_steps (core/optical_flow.py:414-443)
        if (p->gnc_stages < 2 || p->gnc_stages > FRG_MAX_GNC_STAGES)
            return fail(FRG_EINVAL, "gnc_stages must be 0 or in [2, FRG_MAX_GNC_STAGES]");
        for (int s = 0; s < p->gnc_stages; ++s) {
            const double b = p->gnc_schedule[s];
            if (!(b >= 0.0 && b <= 1.0)) return fail(FRG_EINVAL, "gnc_schedule entries must lie in [0, 1]");
            if (s > 0 && !(b >= p->gnc_schedule[s - 1]))
                return fail(FRG_EINVAL, "gnc_schedule must be monotone nondecreasing");
        }
        // np.isclose(x, target) with rtol 1e-5, atol 1e-8
        if (!(std::fabs(p->gnc_schedule[0]) <= 1e-8)) return fail(FRG_EINVAL, "gnc_schedule must start at 0.0");
        if (!(std::fabs(p->gnc_schedule[p->gnc_stages - 1] - 1.0) <= 1e-8 + 1e-5))
            return fail(FRG_EINVAL, "gnc_schedule must end at 1.0");
        if (p->warping_steps < 1) return fail(FRG_EINVAL, "warping_steps must be a positive integer");
    }
    return FRG_OK;
}

int run_xpath(frg_plan* pl, int T, const float* moving, const float* uv_init, double* flow_out, cudaStream_t st);

}  // namespace

extern "C" {

int frg_version(void) { return FRG_ABI_VERSION; }

const char* frg_last_error(void) { return g_last_error.c_str(); }

void frg_plan_destroy(frg_plan* plan)
{
    if (!plan) return;
    for (void* p : plan->allocs) cudaFree(p);
    for (cudaEvent_t e : plan->prof.ev) cudaEventDestroy(e);
    delete plan;
}

long long frg_launch_count(void) { return g_launches.load(); }

int frg_plan_set_profiling(frg_plan* plan, int enable)
{
    if (!plan) return fail(FRG_EINVAL, "plan is NULL");
    plan->prof.on = enable != 0;
    plan->prof.used = 0;
    plan->prof.bytes = 0.0;
    plan->prof.launches = 0;
    return FRG_OK;
}

int frg_plan_profile(frg_plan* plan, long long* sor_launches, double* sor_ms, double* sor_bytes)
{
    if (!plan) return fail(FRG_EINVAL, "plan is NULL");
    double ms = 0.0;
    for (size_t i = 0; i + 1 < plan->prof.used; i += 2) {
        FRG_CUDA(cudaEventSynchronize(plan->prof.ev[i + 1]));
        float t = 0.0f;
        FRG_CUDA(cudaEventElapsedTime(&t, plan->prof.ev[i], plan->prof.ev[i + 1]));
        ms += t;
    }
    if (sor_launches) *sor_launches = plan->prof.launches;
    if (sor_ms) *sor_ms = ms;
    if (sor_bytes) *sor_bytes = plan->prof.bytes;
    return FRG_OK;
}

int frg_plan_create(const frg_params* params, int height, int width, int channels, int max_frames,
                    frg_plan** out)
{
    if (!out) return fail(FRG_EINVAL, "out is NULL");
    *out = nullptr;
    if (height < 2 || width < 2) return fail(FRG_EINVAL, "frame must be at least 2 x 2");
    if (channels < 1 || channels > kMaxK) return fail(FRG_EINVAL, "channels must be in [1, 8]");
    if (max_frames < 1 || max_frames > 65535 / channels)
        return fail(FRG_EINVAL, "max_frames out of range");
    int rc = check_params(params, channels);
    if (rc) return rc;
    if ((rc = ensure_remap_tables())) return rc;

    frg_plan* pl = new frg_plan();
    pl->p = *params;
    pl->H = height;
    pl->W = width;
    pl->K = channels;
    pl->max_T = max_frames;
    for (int k = 0; k < channels; ++k) pl->a_data[k] = (float)params->a_data[k];
    pl->xpath = params->precision == FRG_FP64_REFERENCE || params->a_smooth != 1.0 ||
                params->const_assumption == 2 || params->gnc_stages != 0;
    // the float64 chained SOR serves every float64 level loop without ψ_s or GNC stages: the fp64
    // precision, and census in either precision (the float32 API then rounds its flow)
    pl->dpath = pl->xpath && params->a_smooth == 1.0 && params->gnc_stages == 0;
    const int n_passes = fill_passes(params->iterations, params->update_lag, kGMax, nullptr, 0);
    size_t max_dp64 = 0;
    {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&pl->n_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            pl->n_sms = 1;
    }

    // schedule: core/optical_flow.py:494-518
    const int m = height, n = width;
    const double eta = params->eta;
    int mly = warping_depth(eta, params->levels, m, m);
    int mlx = warping_depth(eta, params->levels, n, n);
    const int max_level = std::min(mlx, mly) * 4;
    mly = std::min(mly, max_level);
    mlx = std::min(mlx, max_level);
    const int top = std::max(mlx, mly);
    int min_level = params->min_level;
    if (top <= min_level) min_level = top - 1;
    if (min_level < 0) min_level = 0;
    pl->min_level = min_level;
    int ph = 0, pw = 0;
    size_t max_dp = 0, max_hw = 0, max_pad = 0;
    for (int i = top; i >= min_level; --i) {
        LevelPlan L;
        L.i = i;
        L.h = (int)std::nearbyint(m * std::pow(eta, (double)std::min(i, mly)));
        L.w = (int)std::nearbyint(n * std::pow(eta, (double)std::min(i, mlx)));
        if (L.h < 1 || L.w < 1) {
            frg_plan_destroy(pl);
            return fail(FRG_EINVAL, "degenerate pyramid level");
        }
        L.top = (i == top);
        L.h_row = (double)m / L.h;
        L.h_col = (double)n / L.w;
        const double sc = (i == min_level) ? 1.0 : std::pow(eta, -0.5 * i);
        L.alpha_x = sc * params->alpha_x;
        L.alpha_y = sc * params->alpha_y;
        L.wx = (float)(L.alpha_x / (L.h_col * L.h_col));
        L.wy = (float)(L.alpha_y / (L.h_row * L.h_row));
        L.g = make_geom(L.h, L.w);
        // the rows-in-registers SOR is the faster kernel wherever it serves (same bits as the
        // diagonal ring; levels taller than 512 rows run it as a cluster of row strips), with
        // all passes of the level chained in one launch
        L.sor_variant = sor_chain_supports(channels, L.g, 1) ? 2 : (sor_regs_supports(channels, L.g) ? 1 : 0);
        const double sig = resize_sigma(m, n, L.h, L.w);
        HostTables tx = make_tables(n, L.w, sig), ty = make_tables(m, L.h, sig);
        if ((rc = upload_tables(pl, tx, L.w, ty, L.h, &L.img))) { frg_plan_destroy(pl); return rc; }
        L.fh = L.top ? m : ph;
        L.fw = L.top ? n : pw;
        const double sigf = resize_sigma(L.fh, L.fw, L.h, L.w);
        HostTables fx = make_tables(L.fw, L.w, sigf), fy = make_tables(L.fh, L.h, sigf);
        if ((rc = upload_tables(pl, fx, L.w, fy, L.h, &L.flow))) { frg_plan_destroy(pl); return rc; }
        if ((rc = dev_alloc(pl, &L.ref, (size_t)channels * L.h * L.w))) { frg_plan_destroy(pl); return rc; }
        if (pl->xpath)
            rc = dev_alloc(pl, &L.wpad64, (size_t)channels * (L.h + 2) * (L.w + 2));
        else
            rc = dev_alloc(pl, &L.wdiag, (size_t)channels * L.g.D * L.g.P);
        if (rc) { frg_plan_destroy(pl); return rc; }
        L.chain64 = pl->dpath && sor_chain64_supports(channels, L.g, n_passes);
        if (L.chain64) {
            if ((rc = dev_alloc(pl, &L.wdiag64, (size_t)2 * channels * L.g.D * L.g.P)) ||
                (rc = dev_alloc(pl, &L.ref64, (size_t)channels * L.h * L.w)) ||
                (rc = dev_alloc(pl, &L.refd64, (size_t)4 * channels * L.h * L.w))) {
                frg_plan_destroy(pl);
                return rc;
            }
            max_dp64 = std::max(max_dp64, (size_t)L.g.D * L.g.P);
        }
        max_dp = std::max(max_dp, (size_t)L.g.D * L.g.P);
        max_hw = std::max(max_hw, (size_t)L.h * L.w);
        max_pad = std::max(max_pad, (size_t)(L.h + 2) * (L.w + 2));
        ph = L.h;
        pw = L.w;
        pl->levels.push_back(L);
    }
    if (min_level > 0) {
        const LevelPlan& Lm = pl->levels.back();
        std::vector<int32_t> sx, sy;
        std::vector<float> wxu, wyu;
        upsample_tables(Lm.w, width, sx, wxu);
        upsample_tables(Lm.h, height, sy, wyu);
        if ((rc = dev_alloc(pl, &pl->up_sx, sx.size())) || (rc = dev_alloc(pl, &pl->up_wx, wxu.size())) ||
            (rc = dev_alloc(pl, &pl->up_sy, sy.size())) || (rc = dev_alloc(pl, &pl->up_wy, wyu.size()))) {
            frg_plan_destroy(pl);
            return rc;
        }
        cudaMemcpy(pl->up_sx, sx.data(), sx.size() * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(pl->up_wx, wxu.data(), wxu.size() * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(pl->up_sy, sy.data(), sy.size() * 4, cudaMemcpyHostToDevice);
        cudaError_t e = cudaMemcpy(pl->up_wy, wyu.data(), wyu.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            frg_plan_destroy(pl);
            return fail(FRG_ECUDA, cudaGetErrorString(e));
        }
        if (pl->xpath &&
            (rc = dev_alloc(pl, &pl->xtmp, (size_t)max_frames * 2 * Lm.h * width))) {
            frg_plan_destroy(pl);
            return rc;
        }
    }

    const size_t T = (size_t)max_frames, K = (size_t)channels;
    const size_t tmp_elems = T * std::max<size_t>(K, 2) * (size_t)height * width;
    if ((rc = dev_alloc(pl, &pl->tmp, tmp_elems)) || (rc = dev_alloc(pl, &pl->f2, T * K * max_hw)) ||
        (rc = dev_alloc(pl, &pl->warped, T * K * max_hw)) ||
        (rc = dev_alloc(pl, &pl->ones, K * (size_t)height * width))) {
        frg_plan_destroy(pl);
        return rc;
    }
    if (pl->xpath) {
        if (params->a_smooth != 1.0 &&
            ((rc = dev_alloc(pl, &pl->xpsis, T * max_pad)) || (rc = dev_alloc(pl, &pl->xsnap, T * 2 * max_pad)))) {
            frg_plan_destroy(pl);
            return rc;
        }
        if (params->precision == FRG_FP32 &&
            (rc = dev_alloc(pl, &pl->xflow, T * 2 * (size_t)height * width))) {
            frg_plan_destroy(pl);
            return rc;
        }
        if ((rc = dev_alloc(pl, &pl->xJ, T * 6 * K * max_pad)) || (rc = dev_alloc(pl, &pl->xwp, T * K * max_pad)) ||
            (rc = dev_alloc(pl, &pl->xdu, T * max_pad)) || (rc = dev_alloc(pl, &pl->xdv, T * max_pad)) ||
            (rc = dev_alloc(pl, &pl->xuv, T * 2 * max_pad)) || (rc = dev_alloc(pl, &pl->xacc[0], T * 2 * max_hw)) ||
            (rc = dev_alloc(pl, &pl->xacc[1], T * 2 * max_hw))) {
            frg_plan_destroy(pl);
            return rc;
        }
        for (int k = 0; k < channels; ++k) pl->a_data64[k] = params->a_data[k];
        if (max_dp64 > 0 && (rc = make_pow_tables(pl, channels))) {
            frg_plan_destroy(pl);
            return rc;
        }
        if (max_dp64 > 0 &&
            ((rc = dev_alloc(pl, &pl->dJ, T * 6 * K * max_dp64)) || (rc = dev_alloc(pl, &pl->dlap, T * 2 * max_dp64)) ||
             (rc = dev_alloc(pl, &pl->dcoef, T * 5 * max_dp64)) || (rc = dev_alloc(pl, &pl->ddu, T * max_dp64)) ||
             (rc = dev_alloc(pl, &pl->ddv, T * max_dp64)))) {
            frg_plan_destroy(pl);
            return rc;
        }
    } else {
        if ((rc = dev_alloc(pl, &pl->J, T * 6 * K * max_dp)) || (rc = dev_alloc(pl, &pl->lap, T * 2 * max_dp)) ||
            (rc = dev_alloc(pl, &pl->coef, T * 5 * max_dp)) || (rc = dev_alloc(pl, &pl->du, T * max_dp)) ||
            (rc = dev_alloc(pl, &pl->dv, T * max_dp)) || (rc = dev_alloc(pl, &pl->uvpad, T * 2 * max_pad)) ||
            (rc = dev_alloc(pl, &pl->uacc[0], T * 2 * max_hw)) ||
            (rc = dev_alloc(pl, &pl->uacc[1], T * 2 * max_hw)) || (rc = dev_alloc(pl, &pl->durm, T * 2 * max_hw))) {
            frg_plan_destroy(pl);
            return rc;
        }
    }
    {
        std::vector<float> ones(K * (size_t)height * width, 1.0f / (float)channels);
        cudaError_t e = cudaMemcpy(pl->ones, ones.data(), ones.size() * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            frg_plan_destroy(pl);
            return fail(FRG_ECUDA, cudaGetErrorString(e));
        }
    }
    *out = pl;
    return FRG_OK;
}

size_t frg_plan_device_bytes(const frg_plan* plan) { return plan ? plan->bytes : 0; }

int frg_schedule(const frg_params* params, int height, int width, int max_levels, int* h, int* w,
                 double* alpha_x, double* alpha_y)
{
    if (!params || height < 2 || width < 2) return -fail(FRG_EINVAL, "bad argument");
    const int m = height, n = width;
    const double eta = params->eta;
    if (!(eta > 0.0 && eta <= 1.0) || params->levels < 1) return -fail(FRG_EINVAL, "bad eta/levels");
    int mly = warping_depth(eta, params->levels, m, m);
    int mlx = warping_depth(eta, params->levels, n, n);
    const int max_level = std::min(mlx, mly) * 4;
    mly = std::min(mly, max_level);
    mlx = std::min(mlx, max_level);
    const int top = std::max(mlx, mly);
    int min_level = params->min_level;
    if (top <= min_level) min_level = top - 1;
    if (min_level < 0) min_level = 0;
    int count = 0;
    for (int i = top; i >= min_level; --i, ++count) {
        if (count >= max_levels) continue;
        if (h) h[count] = (int)std::nearbyint(m * std::pow(eta, (double)std::min(i, mly)));
        if (w) w[count] = (int)std::nearbyint(n * std::pow(eta, (double)std::min(i, mlx)));
        const double sc = (i == min_level) ? 1.0 : std::pow(eta, -0.5 * i);
        if (alpha_x) alpha_x[count] = sc * params->alpha_x;
        if (alpha_y) alpha_y[count] = sc * params->alpha_y;
    }
    return count;
}

int frg_resize_tables(int in_len, int out_len, double sigma, int max_taps, int* idx, float* wt)
{
    if (in_len < 1 || out_len < 1) return -fail(FRG_EINVAL, "bad length");
    HostTables t = make_tables(in_len, out_len, sigma);
    if (t.P > max_taps) return t.P;
    if (idx) for (size_t i = 0; i < t.idx.size(); ++i) idx[i] = t.idx[i];
    if (wt) for (size_t i = 0; i < t.wt.size(); ++i) wt[i] = t.wt[i];
    return t.P;
}

int frg_iteration_passes(int iterations, int update_lag, int max_passes, int* G, int* fold_mode)
{
    if (iterations < 1 || update_lag < 1) return -fail(FRG_EINVAL, "bad iterations/update_lag");
    std::vector<Pass> ps = make_passes(iterations, update_lag);
    for (size_t i = 0; i < ps.size() && (int)i < max_passes; ++i) {
        if (G) G[i] = ps[i].G;
        if (fold_mode) fold_mode[i] = ps[i].fold_mode;
    }
    return (int)ps.size();
}

int frg_plan_num_levels(const frg_plan* plan) { return plan ? (int)plan->levels.size() : 0; }

int frg_plan_set_level_tables(frg_plan* plan, int level, int kind, int taps, const int* ix, const float* wx,
                              const int* iy, const float* wy)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return fail(FRG_EINVAL, "bad level");
    if (kind != 0 && kind != 1) return fail(FRG_EINVAL, "kind must be 0 (image) or 1 (flow)");
    if (!ix || !wx || !iy || !wy) return fail(FRG_EINVAL, "NULL table");
    const LevelPlan& L = plan->levels[level];
    const DevTables& d = kind == 0 ? L.img : L.flow;
    const int in_h = kind == 0 ? plan->H : L.fh, in_w = kind == 0 ? plan->W : L.fw;
    if (taps != d.P) return fail(FRG_EINVAL, "tap count differs from the plan's");
    const size_t nx = (size_t)L.w * taps, ny = (size_t)L.h * taps;
    for (size_t i = 0; i < nx; ++i)
        if (ix[i] < 0 || ix[i] >= in_w) return fail(FRG_EINVAL, "column index out of range");
    for (size_t i = 0; i < ny; ++i)
        if (iy[i] < 0 || iy[i] >= in_h) return fail(FRG_EINVAL, "row index out of range");
    FRG_CUDA(cudaMemcpy(d.ix, ix, nx * 4, cudaMemcpyHostToDevice));
    FRG_CUDA(cudaMemcpy(d.wx, wx, nx * 4, cudaMemcpyHostToDevice));
    FRG_CUDA(cudaMemcpy(d.iy, iy, ny * 4, cudaMemcpyHostToDevice));
    FRG_CUDA(cudaMemcpy(d.wy, wy, ny * 4, cudaMemcpyHostToDevice));
    return FRG_OK;
}

int frg_plan_level_info(const frg_plan* plan, int level, int* h, int* w, double* alpha_x, double* alpha_y)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return fail(FRG_EINVAL, "bad level");
    const LevelPlan& L = plan->levels[level];
    if (h) *h = L.h;
    if (w) *w = L.w;
    if (alpha_x) *alpha_x = L.alpha_x;
    if (alpha_y) *alpha_y = L.alpha_y;
    return FRG_OK;
}

int frg_plan_set_level_tuning(frg_plan* plan, int level, int sor_G, int sor_threads)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return fail(FRG_EINVAL, "bad level");
    LevelPlan& L = plan->levels[level];
    if (L.chain64) {
        // float64 chained SOR: sor_threads = rows per CTA strip (0: chosen from the batch size)
        if (sor_G != 0) return fail(FRG_EINVAL, "the float64 SOR has no pass-length setting (sor_G must be 0)");
        if (sor_threads != 0 && !sor_chain64_rows_ok(L.g, sor_threads))
            return fail(FRG_EINVAL, "sor_threads must be 0, 64, 128 or 256 with at most 8 strips for this level");
        L.rows64 = sor_threads;
        return FRG_OK;
    }
    if (sor_kind(plan->K, L.g) != kSorFused) {
        if (sor_G != 0 || sor_threads != 0) return fail(FRG_EINVAL, "this level does not use the fused SOR kernel");
        return FRG_OK;
    }
    const int gmax = sor_fused_gmax(L.g.P);
    if (sor_G < 0 || sor_G > gmax) return fail(FRG_EINVAL, "sor_G out of range for this level");
    if (sor_threads != 0 && (sor_threads < L.g.P || sor_threads > 2 * kMaxLane || (sor_threads & 31)))
        return fail(FRG_EINVAL, "sor_threads must be 0 or a multiple of 32 in [rows rounded up to 32, 1024]");
    L.sor_G = sor_G;
    L.sor_threads = sor_threads;
    return FRG_OK;
}

int frg_plan_level_tuning(const frg_plan* plan, int level, int* sor_G, int* sor_threads, int* gmax, int* rows)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return fail(FRG_EINVAL, "bad level");
    const LevelPlan& L = plan->levels[level];
    if (L.chain64) {
        if (sor_G) *sor_G = 0;
        if (sor_threads) *sor_threads = L.rows64;
        if (gmax) *gmax = 0;
        if (rows) *rows = L.g.P;
        return FRG_OK;
    }
    const bool fused = sor_kind(plan->K, L.g) == kSorFused;
    if (sor_G) *sor_G = L.sor_G;
    if (sor_threads) *sor_threads = L.sor_threads;
    if (gmax) *gmax = fused ? sor_fused_gmax(L.g.P) : 0;
    if (rows) *rows = L.g.P;
    return FRG_OK;
}

int frg_plan_set_level_variant(frg_plan* plan, int level, int variant)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return fail(FRG_EINVAL, "bad level");
    LevelPlan& L = plan->levels[level];
    if (variant < 0 || variant > 2)
        return fail(FRG_EINVAL, "variant must be 0 (the level's ring / row / global kernel), 1 (rows in registers) "
                                "or 2 (rows in registers, passes chained in one launch)");
    if (variant >= 1 && !sor_regs_supports(plan->K, L.g))
        return fail(FRG_EINVAL, "the rows-in-registers SOR does not serve this level");
    if (variant == 2 && !sor_chain_supports(plan->K, L.g, 1))
        return fail(FRG_EINVAL, "the chained rows-in-registers SOR does not serve this level");
    L.sor_variant = variant;
    return FRG_OK;
}

int frg_plan_level_variant(const frg_plan* plan, int level, int* variant, int* n_variants)
{
    if (!plan || level < 0 || level >= (int)plan->levels.size()) return fail(FRG_EINVAL, "bad level");
    const LevelPlan& L = plan->levels[level];
    if (variant) *variant = L.sor_variant;
    if (n_variants)
        *n_variants = sor_chain_supports(plan->K, L.g, 1) ? 3 : (sor_regs_supports(plan->K, L.g) ? 2 : 1);
    return FRG_OK;
}

int frg_set_reference(frg_plan* pl, const float* fixed, const float* weight, void* stream)
{
    if (!pl || !fixed) return fail(FRG_EINVAL, "plan or fixed is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const int H = pl->H, W = pl->W, K = pl->K;
    const float* wsrc = weight ? weight : pl->ones;
    if (pl->xpath) {
        for (LevelPlan& L : pl->levels) {
            const long long hw = (long long)L.h * L.w, mn = (long long)(L.h + 2) * (L.w + 2);
            FRG_LAUNCH(launch_x_resize_h_f(fixed, 0, 1, (long long)W * K, K, 1, K, H, pl->tmp, L.w, L.img.ix,
                                           L.img.wx, L.img.P, st));
            FRG_LAUNCH(launch_x_resize_v_f(pl->tmp, 1, K, H, L.w, L.ref, 0, hw, L.w, L.h, 0, L.img.iy, L.img.wy,
                                           L.img.P, st));
            FRG_LAUNCH(launch_x_resize_h_f(wsrc, 0, 1, (long long)W * K, K, 1, K, H, pl->tmp, L.w, L.img.ix,
                                           L.img.wx, L.img.P, st));
            FRG_LAUNCH(launch_x_resize_v_d(pl->tmp, 1, K, H, L.w, L.wpad64, 0, mn, L.w + 2, L.h, 2, L.img.iy,
                                           L.img.wy, L.img.P, st));
            if (L.chain64) {
                FRG_LAUNCH(launch_x_pad_to_diag(L.wpad64, K, L.h, L.w, L.g, L.wdiag64, st, pl->a_data64));
                FRG_LAUNCH(launch_x_to_double(L.ref, (long long)K * hw, L.ref64, st));
                FRG_LAUNCH(launch_x_ref_derivs(L.ref64, K, L.h, L.w, L.h_row, L.h_col, L.refd64, st));
            }
        }
        pl->has_ref = true;
        return FRG_OK;
    }
    for (LevelPlan& L : pl->levels) {
        // reference level: resize(fixed) (core/optical_flow.py:519)
        View src = view(fixed, 0, 1, (long long)W * K, K);
        FRG_LAUNCH(launch_resize_h(src, 1, K, H, W, pl->tmp, L.w, L.img.ix, L.img.wx, L.img.P, st));
        FRG_LAUNCH(launch_resize_v(pl->tmp, 1, K, H, L.w, vieww(L.ref, 0, (long long)L.h * L.w, L.w, 1), L.h, 0,
                                 L.img.iy, L.img.wy, L.img.P, st));
        // weight level: resize(weight) (core/optical_flow.py:565-570), diagonal-major
        View wv = view(wsrc, 0, 1, (long long)W * K, K);
        FRG_LAUNCH(launch_resize_h(wv, 1, K, H, W, pl->tmp, L.w, L.img.ix, L.img.wx, L.img.P, st));
        FRG_LAUNCH(launch_resize_v(pl->tmp, 1, K, H, L.w, vieww(pl->f2, 0, (long long)L.h * L.w, L.w, 1), L.h, 0,
                                 L.img.iy, L.img.wy, L.img.P, st));
        FRG_LAUNCH(launch_to_diag(view(pl->f2, 0, (long long)L.h * L.w, L.w, 1), 1, K, L.h, L.w, L.wdiag, 0, L.g,
                                st));
    }
    pl->has_ref = true;
    return FRG_OK;
}

int frg_get_displacement(frg_plan* pl, int T, const float* moving, const float* uv_init, float* flow_out,
                         void* stream)
{
    if (!pl || !moving || !flow_out) return fail(FRG_EINVAL, "NULL argument");
    if (!pl->has_ref) return fail(FRG_EINVAL, "frg_set_reference has not been called");
    if (T < 1 || T > pl->max_T) return fail(FRG_EINVAL, "n_frames out of range for this plan");
    if (pl->p.precision != FRG_FP32)
        return fail(FRG_EINVAL, "this plan computes in fp64: use frg_get_displacement_f64");
    cudaStream_t st = (cudaStream_t)stream;
    const int H = pl->H, W = pl->W, K = pl->K;
    if (pl->xpath) {
        // a_smooth != 1 or census: the reference-order kernels, rounded to float32 at the end
        int rc = run_xpath(pl, T, moving, uv_init, pl->xflow, st);
        if (rc) return rc;
        FRG_LAUNCH(launch_x_to_float(pl->xflow, (long long)T * H * W * 2, flow_out, st));
        return FRG_OK;
    }
    const long long fsz = (long long)H * W * K;
    int cur = 0;
    const LevelPlan* prev = nullptr;
    for (size_t li = 0; li < pl->levels.size(); ++li) {
        const LevelPlan& L = pl->levels[li];
        const int h = L.h, w = L.w;
        const long long hw = (long long)h * w, pad = (long long)(h + 2) * (w + 2);
        const long long dp = (long long)L.g.D * L.g.P;
        // 1. moving level images from full resolution (core/optical_flow.py:520)
        FRG_LAUNCH(launch_resize_h(view(moving, fsz, 1, (long long)W * K, K), T, K, H, W, pl->tmp, w, L.img.ix,
                                 L.img.wx, L.img.P, st));
        FRG_LAUNCH(launch_resize_v(pl->tmp, T, K, H, w, vieww(pl->f2, K * hw, hw, w, 1), h, 0, L.img.iy, L.img.wy,
                                 L.img.P, st));
        // 2. flow at this level with an edge ring (core/optical_flow.py:530-536)
        long long uv_fs;
        if (L.top) {
            uv_fs = 0;  // one field shared by every frame
            if (uv_init) {
                FRG_LAUNCH(launch_resize_h(view(uv_init, 0, 1, (long long)W * 2, 2), 1, 2, H, W, pl->tmp, w,
                                         L.flow.ix, L.flow.wx, L.flow.P, st));
                FRG_LAUNCH(launch_resize_v(pl->tmp, 1, 2, H, w, vieww(pl->uvpad, 0, pad, w + 2, 1), h, 1, L.flow.iy,
                                         L.flow.wy, L.flow.P, st));
            } else {
                FRG_CUDA(cudaMemsetAsync(pl->uvpad, 0, sizeof(float) * 2 * pad, st));
            }
        } else {
            uv_fs = 2 * pad;
            const long long phw = (long long)prev->h * prev->w;
            FRG_LAUNCH(launch_resize_h(view(pl->uacc[cur], 2 * phw, phw, prev->w, 1), T, 2, prev->h, prev->w,
                                     pl->tmp, w, L.flow.ix, L.flow.wx, L.flow.P, st));
            FRG_LAUNCH(launch_resize_v(pl->tmp, T, 2, prev->h, w, vieww(pl->uvpad, 2 * pad, pad, w + 2, 1), h, 1,
                                     L.flow.iy, L.flow.wy, L.flow.P, st));
        }
        View up = view(pl->uvpad, uv_fs, 0, w + 2, 1);
        View vp = view(pl->uvpad + pad, uv_fs, 0, w + 2, 1);
        View f1v = view(L.ref, 0, hw, w, 1);
        View f2v = view(pl->f2, K * hw, hw, w, 1);
        // 3. warp of the moving level by the current flow (core/optical_flow.py:537-542)
        View img2 = f2v;
        if (!L.top) {
            View ui = view(pl->uvpad + (w + 2) + 1, uv_fs, 0, w + 2, 1);
            View vi = view(pl->uvpad + pad + (w + 2) + 1, uv_fs, 0, w + 2, 1);
            FRG_LAUNCH(launch_warp(f2v, f1v, ui, vi, T, K, h, w, (float)L.h_col, (float)L.h_row, 1,
                                 vieww(pl->warped, K * hw, hw, w, 1), st));
            img2 = view(pl->warped, K * hw, hw, w, 1);
        }
        // 4. motion tensor and smoothness constants (core/optical_flow.py:547-563)
        const long long J_fs = 6LL * K * dp;
        FRG_LAUNCH(launch_tensor_lap(f1v, img2, T, K, h, w, (float)L.h_row, (float)L.h_col, pl->p.const_assumption,
                                   pl->J, J_fs, L.g, up, vp, L.wx, L.wy, pl->lap, 2 * dp, st));
        // 5. level solve (core/optical_flow.py:584-606); the fused kernels write the last pass
        // row-major for the median
        const bool fused = sor_kind(K, L.g) == kSorFused || (L.sor_variant >= 1 && sor_regs_supports(K, L.g));
        int rc = solve_level(pl->p.iterations, pl->p.update_lag, pl->J, J_fs, L.wdiag, 0, pl->lap, 2 * dp, pl->du,
                             pl->dv, dp, pl->coef, 5 * dp, T, K, L.g, pl->a_data, L.wx, L.wy, (float)pl->p.omega, st,
                             &pl->prof, pl->durm, pl->durm + (long long)T * hw, hw, L.sor_G, L.sor_threads,
                             L.sor_variant);
        if (rc) return rc;
        // 6. median + accumulate (core/optical_flow.py:607-611)
        const int do_median = std::min(h, w) > 5 ? 1 : 0;
        const bool last = (li + 1 == pl->levels.size());
        ViewW ou, ov;
        if (last && pl->min_level == 0) {
            ou = vieww(flow_out, (long long)H * W * 2, 0, (long long)W * 2, 2);
            ov = vieww(flow_out + 1, (long long)H * W * 2, 0, (long long)W * 2, 2);
        } else {
            const int nxt = cur ^ 1;
            ou = vieww(pl->uacc[nxt], 2 * hw, 0, w, 1);
            ov = vieww(pl->uacc[nxt] + hw, 2 * hw, 0, w, 1);
            cur = nxt;
        }
        if (fused)
            FRG_LAUNCH(launch_median_rm(pl->durm, pl->durm + (long long)T * hw, hw, up, vp, T, h, w, do_median, ou,
                                        ov, st));
        else
            FRG_LAUNCH(launch_median_accum(pl->du, pl->dv, dp, up, vp, T, L.g, do_median, ou, ov, st));
        prev = &L;
    }
    if (pl->min_level > 0) {
        // cv2.resize(w, (n, m), INTER_CUBIC) of the finest computed level (core/optical_flow.py:615-616)
        FRG_LAUNCH(launch_cubic_up<float>(pl->uacc[cur], T, 2, prev->h, prev->w, pl->tmp, flow_out,
                                          (long long)H * W * 2, 1, (long long)W * 2, 2, H, W, pl->up_sx, pl->up_wx,
                                          pl->up_sy, pl->up_wy, st));
    }
    return FRG_OK;
}

}  // extern "C"

namespace {

// GNC stages (core/optical_flow.py:620-770, 909-929) on the reference-order
// kernels.  Each stage re-runs the pyramid from the previous stage's flow
// (flow_out, written by the stage before, read by the next stage's top-level
// resize); each level runs warping_steps rounds of warp (the top level too, so
// the warped frame is float32 everywhere), tensor, compute_flow_gnc from
// du = dv = 0, and the state update u = [median5](u + du) with its border
// rebuilt.  The state is per frame from the start (it changes in place).
int run_xpath_gnc(frg_plan* pl, int T, const float* moving, const float* uv_init, double* flow_out, cudaStream_t st)
{
    const int H = pl->H, W = pl->W, K = pl->K;
    const long long fsz = (long long)H * W * K;
    for (int stage = 0; stage < pl->p.gnc_stages; ++stage) {
        const double beta = pl->p.gnc_schedule[stage];
        int cur = 0;
        const LevelPlan* prev = nullptr;
        for (size_t li = 0; li < pl->levels.size(); ++li) {
            const LevelPlan& L = pl->levels[li];
            const int h = L.h, w = L.w;
            const long long hw = (long long)h * w, mn = (long long)(h + 2) * (w + 2);
            FRG_LAUNCH(launch_x_resize_h_f(moving, fsz, 1, (long long)W * K, K, T, K, H, pl->tmp, w, L.img.ix,
                                           L.img.wx, L.img.P, st));
            FRG_LAUNCH(launch_x_resize_v_f(pl->tmp, T, K, H, w, pl->f2, K * hw, hw, w, h, 0, L.img.iy, L.img.wy,
                                           L.img.P, st));
            if (L.top) {
                if (stage > 0) {
                    FRG_LAUNCH(launch_x_resize_h_d(flow_out, (long long)H * W * 2, 1, (long long)W * 2, 2, T, 2, H,
                                                   pl->tmp, w, L.flow.ix, L.flow.wx, L.flow.P, st));
                } else if (uv_init) {
                    FRG_LAUNCH(launch_x_resize_h_f(uv_init, 0, 1, (long long)W * 2, 2, T, 2, H, pl->tmp, w, L.flow.ix,
                                                   L.flow.wx, L.flow.P, st));
                } else {
                    FRG_CUDA(cudaMemsetAsync(pl->xuv, 0, sizeof(double) * T * 2 * mn, st));
                }
                if (stage > 0 || uv_init)
                    FRG_LAUNCH(launch_x_resize_v_d(pl->tmp, T, 2, H, w, pl->xuv, 2 * mn, mn, w + 2, h, 1, L.flow.iy,
                                                   L.flow.wy, L.flow.P, st));
            } else {
                const long long phw = (long long)prev->h * prev->w;
                FRG_LAUNCH(launch_x_resize_h_d(pl->xacc[cur], 2 * phw, phw, prev->w, 1, T, 2, prev->h, pl->tmp, w,
                                               L.flow.ix, L.flow.wx, L.flow.P, st));
                FRG_LAUNCH(launch_x_resize_v_d(pl->tmp, T, 2, prev->h, w, pl->xuv, 2 * mn, mn, w + 2, h, 1,
                                               L.flow.iy, L.flow.wy, L.flow.P, st));
            }
            const bool last = (li + 1 == pl->levels.size());
            const bool direct = last && pl->min_level == 0;  // the finest level writes flow_out itself
            const int nxt = cur ^ 1;
            double* ou = direct ? flow_out : pl->xacc[nxt];
            double* ov = direct ? flow_out + 1 : pl->xacc[nxt] + hw;
            const long long o_fs = direct ? (long long)H * W * 2 : 2 * hw;
            const long long o_rs = direct ? (long long)W * 2 : w;
            const long long o_cs = direct ? 2 : 1;
            const int do_median = std::min(h, w) > 5 ? 1 : 0;
            for (int ws = 0; ws < pl->p.warping_steps; ++ws) {
                FRG_LAUNCH(launch_x_warp(pl->f2, L.ref, pl->xuv, pl->xuv + mn, 2 * mn, T, K, h, w, L.h_col, L.h_row,
                                         pl->warped, st));
                FRG_LAUNCH(launch_x_tensor(L.ref, pl->warped, T, K, h, w, L.h_row, L.h_col, 1,
                                           pl->p.const_assumption, pl->xJ, st));
                if (pl->p.a_smooth == 1.0) {
                    FRG_LAUNCH(launch_x_sor(pl->xJ, L.wpad64, pl->xuv, pl->xuv + mn, 2 * mn, pl->xdu, pl->xdv,
                                            pl->xwp, T, K, h, w, L.alpha_x, L.alpha_y, L.h_col, L.h_row,
                                            pl->p.iterations, pl->p.update_lag, pl->a_data64, pl->p.omega, beta, st));
                } else {
                    long long n_launch = 0;
                    cudaError_t e = launch_x_sor_smooth(pl->xJ, L.wpad64, pl->xuv, pl->xuv + mn, 2 * mn, pl->xdu,
                                                        pl->xdv, pl->xwp, pl->xpsis, pl->xsnap, T, K, h, w,
                                                        L.alpha_x, L.alpha_y, L.h_col, L.h_row, pl->p.iterations,
                                                        pl->p.update_lag, pl->a_data64, pl->p.a_smooth, pl->p.omega,
                                                        beta, st, &n_launch);
                    g_launches.fetch_add(n_launch, std::memory_order_relaxed);
                    if (e != cudaSuccess)
                        return fail(FRG_ECUDA, std::string("launch_x_sor_smooth: ") + cudaGetErrorString(e));
                }
                // the padded state is needed again unless this is the level's last step
                const int write_ring = ws + 1 < pl->p.warping_steps ? 1 : 0;
                cudaError_t e = launch_x_gnc_update(pl->xdu, pl->xdv, pl->xuv, pl->xuv + mn, 2 * mn, T, h, w,
                                                    do_median, ou, ov, o_fs, o_rs, o_cs, write_ring, st);
                g_launches.fetch_add(1 + write_ring, std::memory_order_relaxed);
                if (e != cudaSuccess)
                    return fail(FRG_ECUDA, std::string("launch_x_gnc_update: ") + cudaGetErrorString(e));
            }
            cur = nxt;
            prev = &L;
        }
        if (pl->min_level > 0) {
            FRG_LAUNCH(launch_cubic_up<double>(pl->xacc[cur], T, 2, prev->h, prev->w, pl->xtmp, flow_out,
                                               (long long)H * W * 2, 1, (long long)W * 2, 2, H, W, pl->up_sx,
                                               pl->up_wx, pl->up_sy, pl->up_wy, st));
        }
    }
    return FRG_OK;
}

// The reference-order level loop (float64 solver), for FP64 plans and for
// a_smooth != 1, census and GNC stages in either precision.
int run_xpath(frg_plan* pl, int T, const float* moving, const float* uv_init, double* flow_out, cudaStream_t st)
{
    if (pl->p.gnc_stages > 0) return run_xpath_gnc(pl, T, moving, uv_init, flow_out, st);
    const int H = pl->H, W = pl->W, K = pl->K;
    const long long fsz = (long long)H * W * K;
    int cur = 0;
    const LevelPlan* prev = nullptr;
    for (size_t li = 0; li < pl->levels.size(); ++li) {
        const LevelPlan& L = pl->levels[li];
        const int h = L.h, w = L.w;
        const long long hw = (long long)h * w, mn = (long long)(h + 2) * (w + 2);
        // moving level images (numba typing of the resize)
        FRG_LAUNCH(launch_x_resize_h_f(moving, fsz, 1, (long long)W * K, K, T, K, H, pl->tmp, w, L.img.ix, L.img.wx,
                                       L.img.P, st));
        FRG_LAUNCH(launch_x_resize_v_f(pl->tmp, T, K, H, w, pl->f2, K * hw, hw, w, h, 0, L.img.iy, L.img.wy, L.img.P,
                                       st));
        // flow with its edge ring
        long long uv_fs;
        if (L.top) {
            uv_fs = 0;
            if (uv_init) {
                FRG_LAUNCH(launch_x_resize_h_f(uv_init, 0, 1, (long long)W * 2, 2, 1, 2, H, pl->tmp, w, L.flow.ix,
                                               L.flow.wx, L.flow.P, st));
                FRG_LAUNCH(launch_x_resize_v_d(pl->tmp, 1, 2, H, w, pl->xuv, 0, mn, w + 2, h, 1, L.flow.iy, L.flow.wy,
                                               L.flow.P, st));
            } else {
                FRG_CUDA(cudaMemsetAsync(pl->xuv, 0, sizeof(double) * 2 * mn, st));
            }
        } else {
            uv_fs = 2 * mn;
            const long long phw = (long long)prev->h * prev->w;
            FRG_LAUNCH(launch_x_resize_h_d(pl->xacc[cur], 2 * phw, phw, prev->w, 1, T, 2, prev->h, pl->tmp, w,
                                           L.flow.ix, L.flow.wx, L.flow.P, st));
            FRG_LAUNCH(launch_x_resize_v_d(pl->tmp, T, 2, prev->h, w, pl->xuv, 2 * mn, mn, w + 2, h, 1, L.flow.iy,
                                           L.flow.wy, L.flow.P, st));
        }
        const float* img2 = pl->f2;
        if (!L.top) {
            FRG_LAUNCH(launch_x_warp(pl->f2, L.ref, pl->xuv, pl->xuv + mn, uv_fs, T, K, h, w, L.h_col, L.h_row,
                                     pl->warped, st));
            img2 = pl->warped;
        }
        if (pl->solver_fn) {
            // the caller's level solver in place of the SOR (core/optical_flow.py:579-606): the
            // tensor in the padded plane layout, then one call per frame once the stream has it
            FRG_LAUNCH(launch_x_tensor(L.ref, img2, T, K, h, w, L.h_row, L.h_col, L.top ? 0 : 1,
                                       pl->p.const_assumption, pl->xJ, st));
            FRG_CUDA(cudaStreamSynchronize(st));
            for (int f = 0; f < T; ++f) {
                const int rc = pl->solver_fn(pl->solver_user, (int)li, f, h + 2, w + 2, K,
                                             pl->xJ + (long long)f * 6 * K * mn, L.wpad64, pl->xuv + f * uv_fs,
                                             pl->xuv + mn + f * uv_fs, L.alpha_x, L.alpha_y, L.h_col, L.h_row,
                                             pl->xdu + (long long)f * mn, pl->xdv + (long long)f * mn);
                if (rc != 0) return fail(FRG_ECALLBACK, "the level solver callback failed");
            }
        } else if (L.chain64) {
            // float64 chained SOR on diagonal-major buffers; the level's last pass writes
            // du, dv into the interiors of the padded xdu, xdv for the median
            const long long dp = (long long)L.g.D * L.g.P;
            const double wx = L.alpha_x / (L.h_col * L.h_col), wy = L.alpha_y / (L.h_row * L.h_row);
            FRG_LAUNCH(launch_x_tensor_diag(L.ref64, L.refd64, L.ref, img2, T, K, h, w, L.h_row, L.h_col,
                                            L.top ? 0 : 1, pl->p.const_assumption, pl->dJ, 6LL * K * dp, L.g, pl->xuv,
                                            pl->xuv + mn, uv_fs, wx, wy, pl->dlap, 2 * dp, st));
            Pass ps[kMaxChain];
            ChainPass cp[kMaxChain];
            const int np = fill_passes(pl->p.iterations, pl->p.update_lag, kGMax, ps, kMaxChain);
            const int its = chain_passes(ps, np, cp);
            const bool timed = pl->prof.on;
            if (timed) {
                int rc = record_event(&pl->prof, st);
                if (rc) return rc;
            }
            const int rows = L.rows64 ? L.rows64 : sor_chain64_default_rows(L.g, T, pl->n_sms);
            FRG_LAUNCH(launch_sor_chain64(pl->dJ, 6LL * K * dp, L.wdiag64, 0, pl->dlap, 2 * dp, pl->dcoef, 5 * dp,
                                          pl->ddu, pl->ddv, dp, T, K, L.g, cp, np, pl->a_data64, wx, wy, pl->p.omega,
                                          st, pl->xdu + (w + 2) + 1, pl->xdv + (w + 2) + 1, mn, w + 2, rows,
                                          pl->pow64));
            if (timed) {
                int rc = record_event(&pl->prof, st);
                if (rc) return rc;
                pl->prof.bytes += 72.0 * its * (double)T * h * w;
                pl->prof.launches += 1;
            }
        } else if (pl->p.a_smooth == 1.0) {
            FRG_LAUNCH(launch_x_tensor(L.ref, img2, T, K, h, w, L.h_row, L.h_col, L.top ? 0 : 1,
                                       pl->p.const_assumption, pl->xJ, st));
            FRG_LAUNCH(launch_x_sor(pl->xJ, L.wpad64, pl->xuv, pl->xuv + mn, uv_fs, pl->xdu, pl->xdv, pl->xwp, T, K,
                                    h, w, L.alpha_x, L.alpha_y, L.h_col, L.h_row, pl->p.iterations,
                                    pl->p.update_lag, pl->a_data64, pl->p.omega, -1.0, st));
        } else {
            FRG_LAUNCH(launch_x_tensor(L.ref, img2, T, K, h, w, L.h_row, L.h_col, L.top ? 0 : 1,
                                       pl->p.const_assumption, pl->xJ, st));
            long long n_launch = 0;
            cudaError_t e = launch_x_sor_smooth(pl->xJ, L.wpad64, pl->xuv, pl->xuv + mn, uv_fs, pl->xdu, pl->xdv,
                                                pl->xwp, pl->xpsis, pl->xsnap, T, K, h, w, L.alpha_x, L.alpha_y,
                                                L.h_col, L.h_row, pl->p.iterations, pl->p.update_lag, pl->a_data64,
                                                pl->p.a_smooth, pl->p.omega, -1.0, st, &n_launch);
            g_launches.fetch_add(n_launch, std::memory_order_relaxed);
            if (e != cudaSuccess) return fail(FRG_ECUDA, std::string("launch_x_sor_smooth: ") + cudaGetErrorString(e));
        }
        const int do_median = std::min(h, w) > 5 ? 1 : 0;
        const bool last = (li + 1 == pl->levels.size());
        if (last && pl->min_level == 0) {
            FRG_LAUNCH(launch_x_median_accum(pl->xdu, pl->xdv, pl->xuv, pl->xuv + mn, uv_fs, T, h, w, do_median,
                                             flow_out, flow_out + 1, (long long)H * W * 2, (long long)W * 2, 2, st));
        } else {
            const int nxt = cur ^ 1;
            FRG_LAUNCH(launch_x_median_accum(pl->xdu, pl->xdv, pl->xuv, pl->xuv + mn, uv_fs, T, h, w, do_median,
                                             pl->xacc[nxt], pl->xacc[nxt] + hw, 2 * hw, w, 1, st));
            cur = nxt;
        }
        prev = &L;
    }
    if (pl->min_level > 0) {
        FRG_LAUNCH(launch_cubic_up<double>(pl->xacc[cur], T, 2, prev->h, prev->w, pl->xtmp, flow_out,
                                           (long long)H * W * 2, 1, (long long)W * 2, 2, H, W, pl->up_sx, pl->up_wx,
                                           pl->up_sy, pl->up_wy, st));
    }
    return FRG_OK;
}

}  // namespace

extern "C" {

int frg_get_displacement_f64(frg_plan* pl, int T, const float* moving, const float* uv_init, double* flow_out,
                             void* stream)
{
    if (!pl || !moving || !flow_out) return fail(FRG_EINVAL, "NULL argument");
    if (!pl->has_ref) return fail(FRG_EINVAL, "frg_set_reference has not been called");
    if (T < 1 || T > pl->max_T) return fail(FRG_EINVAL, "n_frames out of range for this plan");
    if (pl->p.precision != FRG_FP64_REFERENCE)
        return fail(FRG_EINVAL, "this plan computes in fp32: use frg_get_displacement");
    return run_xpath(pl, T, moving, uv_init, flow_out, (cudaStream_t)stream);
}

int frg_pow_f64(long long n, const double* x, double b, double* out, void* stream)
{
    if (n < 0 || (n > 0 && (!x || !out))) return fail(FRG_EINVAL, "bad argument");
    int rc = ensure_remap_tables();
    if (rc) return rc;
    FRG_LAUNCH(launch_pow64(n, x, b, out, (cudaStream_t)stream));
    return FRG_OK;
}

int frg_imregister(int n_frames, int height, int width, int channels, const float* frames, const float* flow,
                   const float* reference, int cubic, float* out, void* stream)
{
    if (!frames || !flow || !reference || !out) return fail(FRG_EINVAL, "NULL argument");
    if (n_frames < 1 || n_frames > 65535 || height < 1 || width < 1 || channels < 1)
        return fail(FRG_EINVAL, "bad shape");
    int rc = ensure_remap_tables();
    if (rc) return rc;
    const long long H = height, W = width, K = channels;
    View f2 = view(frames, H * W * K, 1, W * K, K);
    View f1 = view(reference, 0, 1, W * K, K);
    View u = view(flow, H * W * 2, 0, W * 2, 2);
    View v = view(flow + 1, H * W * 2, 0, W * 2, 2);
    ViewW o = vieww(out, H * W * K, 1, W * K, K);
    FRG_LAUNCH(launch_warp(f2, f1, u, v, n_frames, channels, height, width, 1.0f, 1.0f, cubic ? 1 : 0, o,
                         (cudaStream_t)stream));
    return FRG_OK;
}

int frg_level_solve(int m, int n, int K, const float* J, const float* weight, const float* u, const float* v,
                    double alpha_x, double alpha_y, int iterations, int update_lag, const double* a_data,
                    double a_smooth, double hx, double hy, double omega, float* du, float* dv, void* stream)
{
    if (!J || !weight || !u || !v || !a_data || !du || !dv) return fail(FRG_EINVAL, "NULL argument");
    if (m < 3 || n < 3 || K < 1 || K > kMaxK) return fail(FRG_EINVAL, "bad shape");
    if (iterations < 1 || update_lag < 1) return fail(FRG_EINVAL, "iterations and update_lag must be >= 1");
    if (a_smooth != 1.0) return fail(FRG_EUNSUPPORTED, "a_smooth != 1 is not supported by the GB300 backend");
    const int h = m - 2, w = n - 2;
    DiagGeom g = make_geom(h, w);
    cudaStream_t st = (cudaStream_t)stream;
    const long long dp = (long long)g.D * g.P;
    const long long mn = (long long)m * n;
    float* scratch = nullptr;
    const size_t elems = (size_t)(6 * K + K + 2 + 5 + 2) * dp;
    FRG_CUDA(cudaMallocAsync((void**)&scratch, elems * sizeof(float), st));
    float* Jd = scratch;
    float* Wd = Jd + 6LL * K * dp;
    float* lap = Wd + (long long)K * dp;
    float* coef = lap + 2 * dp;
    float* dud = coef + 5 * dp;
    float* dvd = dud + dp;
    int rc = FRG_OK;
    float ad[kMaxK];
    for (int k = 0; k < K; ++k) ad[k] = (float)a_data[k];
    const float wx = (float)(alpha_x / (hx * hx)), wy = (float)(alpha_y / (hy * hy));
    auto run = [&]() -> int {
        // J arrays (m, n, K) channel-last; interior starts at (1, 1)
        for (int q = 0; q < 6; ++q)
            FRG_LAUNCH(launch_to_diag(view(J + q * mn * K + (n + 1) * (long long)K, 0, 1, (long long)n * K, K), 1, K,
                                    h, w, Jd + q * K * dp, 0, g, st));
        FRG_LAUNCH(launch_to_diag(view(weight + (n + 1) * (long long)K, 0, 1, (long long)n * K, K), 1, K, h, w, Wd,
                                0, g, st));
        FRG_LAUNCH(launch_lap(view(u, 0, 0, n, 1), view(v, 0, 0, n, 1), 1, h, w, wx, wy, lap, 2 * dp, g, st));
        int r = solve_level(iterations, update_lag, Jd, 0, Wd, 0, lap, 0, dud, dvd, 0, coef, 0, 1, K, g, ad, wx, wy,
                            (float)omega, st, nullptr, nullptr, nullptr, 0, 0, 0,
                            sor_chain_supports(K, g, 1) ? 2 : (sor_regs_supports(K, g) ? 1 : 0));
        if (r) return r;
        FRG_LAUNCH(launch_from_diag(dud, 0, 1, 1, g, vieww(du, 0, 0, n, 1), 1, 2, st));
        FRG_LAUNCH(launch_from_diag(dvd, 0, 1, 1, g, vieww(dv, 0, 0, n, 1), 1, 2, st));
        return FRG_OK;
    };
    rc = run();
    cudaError_t e = cudaFreeAsync(scratch, st);
    if (rc == FRG_OK && e != cudaSuccess) return fail(FRG_ECUDA, cudaGetErrorString(e));
    return rc;
}

int frg_level_solve_f64(int m, int n, int K, const double* J, const double* weight, const double* u, const double* v,
                        double alpha_x, double alpha_y, int iterations, int update_lag, const double* a_data,
                        double a_smooth, double hx, double hy, double omega, double gnc_beta, double* du, double* dv,
                        void* stream)
{
    if (!J || !weight || !u || !v || !a_data || !du || !dv) return fail(FRG_EINVAL, "NULL argument");
    if (m < 3 || n < 3 || K < 1 || K > kMaxK) return fail(FRG_EINVAL, "bad shape");
    if (iterations < 1 || update_lag < 1) return fail(FRG_EINVAL, "iterations and update_lag must be >= 1");
    if (!(a_smooth > 0.0)) return fail(FRG_EINVAL, "a_smooth must be > 0");
    if (gnc_beta > 1.0) return fail(FRG_EINVAL, "gnc_beta must lie in [0, 1] (negative: no GNC)");
    const int h = m - 2, w = n - 2;
    const long long mn = (long long)m * n;
    const bool smooth = a_smooth != 1.0;
    cudaStream_t st = (cudaStream_t)stream;
    double* scratch = nullptr;
    const size_t elems = (size_t)(6 * K + 2 * K + (smooth ? 3 : 0)) * mn;
    FRG_CUDA(cudaMallocAsync((void**)&scratch, elems * sizeof(double), st));
    double* Jp = scratch;              // (6, K, mn)
    double* Wp = Jp + 6LL * K * mn;    // (K, mn)
    double* wp = Wp + (long long)K * mn;
    double* psis = wp + (long long)K * mn;
    double* snap = psis + mn;
    auto run = [&]() -> int {
        FRG_LAUNCH(launch_x_hwk_to_planes(J, 6, mn, K, Jp, st));
        FRG_LAUNCH(launch_x_hwk_to_planes(weight, 1, mn, K, Wp, st));
        if (!smooth) {
            FRG_LAUNCH(launch_x_sor(Jp, Wp, u, v, 0, du, dv, wp, 1, K, h, w, alpha_x, alpha_y, hx, hy, iterations,
                                    update_lag, a_data, omega, gnc_beta, st));
        } else {
            long long n_launch = 0;
            cudaError_t e = launch_x_sor_smooth(Jp, Wp, u, v, 0, du, dv, wp, psis, snap, 1, K, h, w, alpha_x,
                                                alpha_y, hx, hy, iterations, update_lag, a_data, a_smooth, omega,
                                                gnc_beta, st, &n_launch);
            g_launches.fetch_add(n_launch, std::memory_order_relaxed);
            if (e != cudaSuccess) return fail(FRG_ECUDA, std::string("launch_x_sor_smooth: ") + cudaGetErrorString(e));
        }
        return FRG_OK;
    };
    const int rc = run();
    cudaError_t e = cudaFreeAsync(scratch, st);
    if (rc == FRG_OK && e != cudaSuccess) return fail(FRG_ECUDA, cudaGetErrorString(e));
    return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// frg_level_solve_noalloc: frg_level_solve for callers that cannot allocate
// device memory.  Its scratch is this file-scope device array, a fixed 8 MiB
// that every GPU loading the library keeps until the process exits.  Host code
// must not use `g_noalloc_scratch` as a pointer (it names the host-side shadow);
// the device address comes from cudaGetSymbolAddress, looked up once per device
// with that device current, on the first call on that device.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocFloats = size_t(2) << 20;  // 2 Mi floats = 8 MiB
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocFloats];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
float* g_noalloc_ptr[kMaxDevices] = {nullptr};

int noalloc_scratch(float** out)
{
    int dev = -1;
    FRG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(FRG_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        FRG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = (float*)p;
    }
    *out = g_noalloc_ptr[dev];
    return FRG_OK;
}

}  // namespace

extern "C" {

size_t frg_level_solve_noalloc_capacity(void) { return kNoAllocFloats * sizeof(float); }

int frg_level_solve_noalloc(int m, int n, int K, const float* J, const float* weight, const float* u, const float* v,
                            double alpha_x, double alpha_y, int iterations, int update_lag, const double* a_data,
                            double a_smooth, double hx, double hy, double omega, float* du, float* dv, void* stream)
{
    if (!J || !weight || !u || !v || !a_data || !du || !dv) return fail(FRG_EINVAL, "NULL argument");
    if (m < 3 || n < 3 || K < 1 || K > kMaxK) return fail(FRG_EINVAL, "bad shape");
    if (iterations < 1 || update_lag < 1) return fail(FRG_EINVAL, "iterations and update_lag must be >= 1");
    if (a_smooth != 1.0) return fail(FRG_EUNSUPPORTED, "a_smooth != 1 is not supported by the GB300 backend");
    const int h = m - 2, w = n - 2;
    DiagGeom g = make_geom(h, w);
    const long long dp = (long long)g.D * g.P;
    const size_t elems = (size_t)(6 * K + K + 2 + 5 + 2) * (size_t)dp;
    if (elems > kNoAllocFloats)
        return fail(FRG_EINVAL, "level too large for the 8 MiB scratch of frg_level_solve_noalloc: needs " +
                                    std::to_string(elems * sizeof(float)) + " bytes ((7K+9)*(h+w-1)*ceil32(h) floats)");
    float* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const long long mn = (long long)m * n;
    float* Jd = scratch;
    float* Wd = Jd + 6LL * K * dp;
    float* lap = Wd + (long long)K * dp;
    float* coef = lap + 2 * dp;
    float* dud = coef + 5 * dp;
    float* dvd = dud + dp;
    float ad[kMaxK];
    for (int k = 0; k < K; ++k) ad[k] = (float)a_data[k];
    const float wx = (float)(alpha_x / (hx * hx)), wy = (float)(alpha_y / (hy * hy));
    // Every scratch element read below is first written in this call: to_diag
    // and lap fill all pixels of the level, and the first fold sets du = dv = 0.
    for (int q = 0; q < 6; ++q)
        FRG_LAUNCH(launch_to_diag(view(J + q * mn * K + (n + 1) * (long long)K, 0, 1, (long long)n * K, K), 1, K, h,
                                  w, Jd + q * K * dp, 0, g, st));
    FRG_LAUNCH(launch_to_diag(view(weight + (n + 1) * (long long)K, 0, 1, (long long)n * K, K), 1, K, h, w, Wd, 0, g,
                              st));
    FRG_LAUNCH(launch_lap(view(u, 0, 0, n, 1), view(v, 0, 0, n, 1), 1, h, w, wx, wy, lap, 2 * dp, g, st));
    // The kernels frg_level_solve runs for the same level (solve_level with the
    // variant it picks), so both give the same bits, with the passes generated
    // into stack arrays instead of host containers: the chained SOR (K <= 4,
    // at most kMaxChain passes), else the rows-in-registers SOR pass by pass
    // (K <= 4), else (K > 4) the fold kernel at each group start and the
    // row-per-thread SOR.  Every level within the scratch limit has at most
    // 512 rows (one of 513 rows needs over 8 MiB at any K); the global-memory
    // wavefront below only keeps the branch complete.
    const bool regs = sor_regs_supports(K, g);
    Pass ps[kMaxChain];
    const int n_passes = fill_passes(iterations, update_lag, kGMax, ps, kMaxChain);
    if (n_passes <= kMaxChain && sor_chain_supports(K, g, n_passes)) {
        ChainPass cp[kMaxChain];
        chain_passes(ps, n_passes, cp);
        FRG_LAUNCH(launch_sor_chain(Jd, 0, Wd, 0, lap, 0, coef, 0, dud, dvd, 0, 1, K, g, cp, n_passes, ad, wx, wy,
                                    (float)omega, st, nullptr, nullptr, 0));
    } else {
        for (int t = 0; t < iterations;) {
            const bool tick = ((t + 1) % update_lag) == 0;
            int end = t + 1;
            while (end < iterations && ((end + 1) % update_lag) != 0) ++end;
            const int mode = (t == 0 ? 1 : 0) | (tick ? 2 : 0);
            for (int s = t; s < end; s += kGMax) {
                const int G = std::min(kGMax, end - s);
                const int pass_mode = s == t ? mode : -1;
                if (regs) {
                    const int store = (s == t && s + kGMax < end) ? 1 : 0;
                    FRG_LAUNCH(launch_sor_regs(Jd, 0, Wd, 0, lap, 0, coef, 0, dud, dvd, 0, 1, K, g, G, pass_mode,
                                               store, ad, wx, wy, (float)omega, st));
                } else {
                    if (pass_mode >= 0)
                        FRG_LAUNCH(launch_fold(Jd, 0, Wd, 0, lap, 0, dud, dvd, 0, coef, 0, 1, K, g, ad, pass_mode, wx,
                                               wy, st));
                    if (g.P <= kMaxLane)
                        FRG_LAUNCH(launch_sor(coef, 0, dud, dvd, 0, 1, g, G, wy, wx, (float)omega, st));
                    else
                        FRG_LAUNCH(launch_sor_global(coef, 0, dud, dvd, 0, 1, g, G, wy, wx, (float)omega, st));
                }
            }
            t = end;
        }
    }
    FRG_LAUNCH(launch_from_diag(dud, 0, 1, 1, g, vieww(du, 0, 0, n, 1), 1, 2, st));
    FRG_LAUNCH(launch_from_diag(dvd, 0, 1, 1, g, vieww(dv, 0, 0, n, 1), 1, 2, st));
    return FRG_OK;
}

int frg_resize(int n_planes, int ih, int iw, const float* src, int oh, int ow, float* dst, void* stream)
{
    if (!src || !dst || n_planes < 1 || ih < 1 || iw < 1 || oh < 1 || ow < 1) return fail(FRG_EINVAL, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    const double sig = resize_sigma(ih, iw, oh, ow);
    HostTables tx = make_tables(iw, ow, sig), ty = make_tables(ih, oh, sig);
    const size_t tb = (tx.idx.size() + tx.wt.size() + ty.idx.size() + ty.wt.size()) * 4;
    const size_t tmpb = (size_t)n_planes * ih * ow * 4;
    char* buf = nullptr;
    FRG_CUDA(cudaMallocAsync((void**)&buf, tb + tmpb, st));
    int32_t* ix = (int32_t*)buf;
    float* wx = (float*)(ix + tx.idx.size());
    int32_t* iy = (int32_t*)(wx + tx.wt.size());
    float* wy = (float*)(iy + ty.idx.size());
    float* tmp = wy + ty.wt.size();
    auto run = [&]() -> int {
        FRG_CUDA(cudaMemcpyAsync(ix, tx.idx.data(), tx.idx.size() * 4, cudaMemcpyHostToDevice, st));
        FRG_CUDA(cudaMemcpyAsync(wx, tx.wt.data(), tx.wt.size() * 4, cudaMemcpyHostToDevice, st));
        FRG_CUDA(cudaMemcpyAsync(iy, ty.idx.data(), ty.idx.size() * 4, cudaMemcpyHostToDevice, st));
        FRG_CUDA(cudaMemcpyAsync(wy, ty.wt.data(), ty.wt.size() * 4, cudaMemcpyHostToDevice, st));
        FRG_LAUNCH(launch_resize_h(view(src, 0, (long long)ih * iw, iw, 1), 1, n_planes, ih, iw, tmp, ow, ix, wx, tx.P,
                                 st));
        FRG_LAUNCH(launch_resize_v(tmp, 1, n_planes, ih, ow, vieww(dst, 0, (long long)oh * ow, ow, 1), oh, 0, iy, wy,
                                 ty.P, st));
        // the host vectors must outlive the asynchronous copies
        FRG_CUDA(cudaStreamSynchronize(st));
        return FRG_OK;
    };
    int rc = run();
    cudaError_t e = cudaFreeAsync(buf, st);
    if (rc == FRG_OK && e != cudaSuccess) return fail(FRG_ECUDA, cudaGetErrorString(e));
    return rc;
}

int frg_motion_tensor(int h, int w, const float* f1, const float* f2, double hy, double hx, int gray, float* out,
                      void* stream)
{
    if (!f1 || !f2 || !out || h < 1 || w < 1) return fail(FRG_EINVAL, "bad argument");
    if (h > 4096 || w > 4096) return fail(FRG_EINVAL, "plane too large");
    if (gray != 0 && gray != 1)
        return fail(FRG_EUNSUPPORTED, "frg_motion_tensor computes gc or gray; census runs inside a plan");
    cudaStream_t st = (cudaStream_t)stream;
    DiagGeom g = make_geom(h, w);
    const long long dp = (long long)g.D * g.P;
    float* Jd = nullptr;
    FRG_CUDA(cudaMallocAsync((void**)&Jd, 6 * dp * sizeof(float), st));
    auto run = [&]() -> int {
        FRG_LAUNCH(launch_tensor(view(f1, 0, 0, w, 1), view(f2, 0, 0, w, 1), 1, 1, h, w, (float)hy, (float)hx,
                               gray ? 1 : 0, Jd, 0, g, st));
        const long long pad = (long long)(h + 2) * (w + 2);
        FRG_LAUNCH(launch_from_diag(Jd, 0, 1, 6, g, vieww(out, 0, pad, w + 2, 1), 1, 1, st));
        return FRG_OK;
    };
    int rc = run();
    cudaError_t e = cudaFreeAsync(Jd, st);
    if (rc == FRG_OK && e != cudaSuccess) return fail(FRG_ECUDA, cudaGetErrorString(e));
    return rc;
}

int frg_median5(int h, int w, const float* src, float* dst, void* stream)
{
    if (!src || !dst || h < 3 || w < 3) return fail(FRG_EINVAL, "bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    const long long pad = (long long)(h + 2) * (w + 2);
    float* buf = nullptr;
    FRG_CUDA(cudaMallocAsync((void**)&buf, pad * sizeof(float), st));
    float* zeros = buf;
    auto run = [&]() -> int {
        FRG_CUDA(cudaMemsetAsync(zeros, 0, pad * sizeof(float), st));
        View z = view(zeros, 0, 0, w + 2, 1);
        // the pipeline's median kernel on one plane; the v output duplicates u
        // and goes to the same destination
        FRG_LAUNCH(launch_median_rm(src, src, 0, z, z, 1, h, w, 1, vieww(dst, 0, 0, w, 1), vieww(dst, 0, 0, w, 1),
                                    st));
        return FRG_OK;
    };
    int rc = run();
    cudaError_t e = cudaFreeAsync(buf, st);
    if (rc == FRG_OK && e != cudaSuccess) return fail(FRG_ECUDA, cudaGetErrorString(e));
    return rc;
}

int frg_host_register(void* ptr, long long bytes)
{
    if (!ptr || bytes <= 0) return fail(FRG_EINVAL, "bad argument");
    const cudaError_t e = cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();  // a refusal is reported here, not by the next launch
        return fail(FRG_ECUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
    }
    return FRG_OK;
}

int frg_host_unregister(void* ptr)
{
    if (!ptr) return fail(FRG_EINVAL, "bad argument");
    const cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(FRG_ECUDA, std::string("cudaHostUnregister: ") + cudaGetErrorString(e));
    }
    return FRG_OK;
}

int frg_plan_set_level_solver(frg_plan* pl, frg_level_solver_fn fn, void* user)
{
    if (!pl) return fail(FRG_EINVAL, "NULL plan");
    if (!pl->xpath || pl->p.gnc_stages > 0)
        return fail(FRG_EUNSUPPORTED, "a host level solver needs a float64 plan without GNC stages");
    pl->solver_fn = fn;
    pl->solver_user = fn ? user : nullptr;
    return FRG_OK;
}

int frg_median5_f64(int h, int w, const double* src, double* dst, void* stream)
{
    if (!src || !dst || h < 3 || w < 3) return fail(FRG_EINVAL, "bad argument");
    FRG_LAUNCH(launch_x_median5_plane(src, h, w, dst, (cudaStream_t)stream));
    return FRG_OK;
}

}  // extern "C"

// Host helpers shared with frg_diff_api.cu (declared in frg_internal.h).
namespace frg {
int host_fail(int code, const std::string& msg) { return fail(code, msg); }
void host_count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int host_warping_depth(double eta, int levels, int m, int n) { return warping_depth(eta, levels, m, n); }
double host_resize_sigma(int ih, int iw, int oh, int ow) { return resize_sigma(ih, iw, oh, ow); }
int host_make_tables(int in_len, int out_len, double sigma, std::vector<int32_t>& idx, std::vector<float>& wt)
{
    HostTables t = make_tables(in_len, out_len, sigma);
    idx = std::move(t.idx);
    wt = std::move(t.wt);
    return t.P;
}
}  // namespace frg
