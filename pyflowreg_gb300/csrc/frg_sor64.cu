// Exact-order chained SOR in float64 (the parity precision).
//
// compute_flow (core/level_solver.py:158-369) sweeps columns outer, rows
// inner, in place, in float64.  Float32 arithmetic moves the flow by up to
// ~0.7 px against it: the 1/32-pixel warp of the next level turns rounding
// differences into different samples.  With every solver operation rounded to
// 44 mantissa bits the flow still moves by 2e-3 px; at 48 bits by 1e-8 px.
// So the parity path computes in float64, and on GB300, whose float64 pipe
// issues at about 1/64 of the float32 rate, it is bound by float64
// instructions: this kernel keeps the instruction count per update at the
// minimum (14 float64 operations per pixel update, the coefficients folded
// once per pass) and everything else off the float64 pipe.
//
// Schedule: that of k_sor_chain (frg_sor.cu).  Row r's local time is
// tau = s - r; pass p occupies tau in [start_p, start_p + span_p), pixel (r, c)
// of pipelined iteration gi is updated at tau = start_p + c + 2 gi, and every
// neighbour value an update reads was produced one step earlier, so it stays
// in registers (left, right, own) or comes from the neighbouring row through a
// warp shuffle (up, down) or the two-parity exchange buffer (warp edges).
// Each pixel's five coefficients (A12, BU, BV, omega/den_u, omega/den_v) are
// folded once per pass when the pixel enters and wait in a shared-memory ring
// of 2G - 1 slots until its last update of the pass.
//
// One thread per row, at most 256, 128 or 64 rows per CTA (a launch choice:
// the shorter strips fit three or six CTAs per SM, or spread a single frame
// over more SMs); taller levels run as a thread-block cluster of row strips
// whose edge rows exchange their values through distributed shared memory,
// with a cluster barrier per step.
#include "frg_internal.h"
#include "frg_dpow.cuh"

#include <cooperative_groups.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

namespace frg {

// The tables of dpow_tab, from the host's long double log2 / exp2 (extended or
// quadruple precision), rounded to double once.
cudaError_t upload_dpow_tables()
{
    static std::mutex mu;
    static std::set<int> done;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(dev)) return cudaSuccess;
    double lt[3 * kDpowLogN], et[kDpowExpN];
    const long double two42 = 4398046511104.0L;
    for (int j = 0; j < kDpowLogN; ++j) {
        const double c = 1.0 + (2.0 * j + 1.0) / 512.0;  // exact
        const double inv = 1.0 / c;
        const long double L = -log2l((long double)inv);   // in [0, 1)
        const double Lhi = (double)(nearbyintl(L * two42) / two42);
        const double Llo = (double)(L - (long double)Lhi);
        const long long L42 = (long long)nearbyintl(L * two42);  // Lhi 2^42, below 2^42
        lt[3 * j] = inv;
        std::memcpy(&lt[3 * j + 1], &L42, sizeof(L42));
        lt[3 * j + 2] = Llo;
    }
    for (int i = 0; i < kDpowExpN; ++i) et[i] = (double)exp2l((long double)i / (long double)kDpowExpN);
    if ((e = cudaMemcpyToSymbol(g_dpow_log, lt, sizeof(lt))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(g_dpow_exp, et, sizeof(et))) != cudaSuccess) return e;
    done.insert(dev);
    return cudaSuccess;
}

// dpow_b's table for exponent b: T(e, j) = 2^(e b) (1 / inv_j)^b in long double,
// split into a double and the double of the remainder; inv_j as the device's
// log table holds it.
bool make_pow_table(double b, double2* tab, PowTab64* pt)
{
    if (!(b >= -1.0 && b <= 1.0)) return false;
    const long double lb = b;
    long double B[256];
    for (int j = 0; j < 256; ++j) {
        const double c = 1.0 + (2.0 * j + 1.0) / 512.0;  // exact
        const double inv = 1.0 / c;
        B[j] = exp2l(-lb * log2l((long double)inv));
    }
    for (int e = 0; e < kPowTabN / 256; ++e) {
        const long double A = exp2l((long double)(e + kPowEMin) * lb);
        for (int j = 0; j < 256; ++j) {
            const long double v = A * B[j];
            const double hi = (double)v;
            tab[e * 256 + j] = make_double2(hi, (double)(v - (long double)hi));
        }
    }
    // binomial coefficients C(b, n) = C(b, n - 1) (b - n + 1) / n
    long double c = lb, cn[7];
    for (int n = 2; n <= 6; ++n) cn[n] = c = c * (lb - (n - 1)) / n;
    pt->c2 = (double)cn[2];
    pt->c3 = (double)cn[3];
    pt->c4 = (float)cn[4];
    pt->c5 = (float)cn[5];
    pt->c6 = (float)cn[6];
    return true;
}

namespace {

__global__ void k_pow64(long long n, const double* __restrict__ x, double b, PowTab64 P, double* __restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = dpow_b(x[i], b, P);
}

}  // namespace

cudaError_t launch_pow64(long long n, const double* x, double b, double* out, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    if ((n + 255) / 256 > 0x7fffffffLL) return cudaErrorInvalidValue;
    PowTab64 P;
    std::vector<double2> tab(kPowTabN);
    double2* dt = nullptr;
    if (make_pow_table(b, tab.data(), &P)) {
        // stream-ordered: the copy from pageable memory returns once the table is staged
        cudaError_t e = cudaMallocAsync((void**)&dt, sizeof(double2) * kPowTabN, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dt, tab.data(), sizeof(double2) * kPowTabN, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            if (dt) cudaFreeAsync(dt, st);
            return e;
        }
        P.t = dt;
    }
    k_pow64<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, b, P, out);
    cudaError_t e = cudaGetLastError();
    if (dt) {
        const cudaError_t f = cudaFreeAsync(dt, st);
        if (e == cudaSuccess) e = f;
    }
    return e;
}

namespace {

constexpr int kLane64 = 256;       // most rows (threads) per CTA
constexpr int kG64 = kGMax;        // iterations pipelined per pass, as a template maximum
constexpr int kSmem64 = 232448;    // 227 KB of dynamic shared memory per CTA
constexpr int kMaxStrips64 = 16;   // cluster size (over 8: the non-portable opt-in)
constexpr int kPortableStrips = 8;

struct Sor64Args {
    const double* J;    // [6][K][D*P] per frame: J11, J22, J33 + 1e-5, 2 J12, 2 J13, 2 J23
    long long J_fs;
    const double* W;    // [2][K][D*P] per frame, W then W * a_data (W_fs 0: shared by all frames)
    long long W_fs;
    const double* lap;  // [2][D*P]: the u- and v-parts of the smoothness numerator from u, v
    long long lap_fs;
    double* coef;       // [5][D*P]: folded coefficients of passes that continue a group
    long long coef_fs;
    double* du;         // [D*P] pass-to-pass state
    double* dv;
    long long st_fs;
    double* out_du;     // final pass: du, dv at out + r * out_rs + c (frame stride out_fs)
    double* out_dv;
    long long out_fs;
    int out_rs;
    DiagGeom g;
    double wa, wb;      // smoothness weights of the row neighbours (y) and the column neighbours (x)
    double wsum;        // ((wx + wx) + wy) + wy, the reference's order
    double omega, one_m_omega;
    double a_m1[kMaxK];  // a_data - 1
    PowTab64 pw[kMaxK];  // the power's table per channel (null table: the general power)
    int nc;              // row strips (CTAs) per frame
};

struct Chain64Table {
    int n;
    int pk[kMaxChain];  // G << 8 | store << 3 | coef << 2 | tick << 1 | zero
};

constexpr int kPkZero = 1, kPkTick = 2, kPkCoef = 4, kPkStore = 8;

// The fold's inputs of one pixel (J, W, lap; or the stored coefficients),
// loaded at the start of the step whose end folds them: a step of float64
// work takes several microseconds, far longer than the loads.
template <int K>
struct FoldIn64 {
    double j[6 * K];
    double w[K];
    double lu, lv;
};

// Pass-start state, prefetched two steps ahead: du, dv of pixel (r, c) entering
// the ring and of pixel (r + 1, c - 1) below its left neighbour.
struct Pre64 {
    double du, dv, nu, nv;
};

struct Coef64 {
    double A12, BU, BV, iDu, iDv;
};

// 1 / x for a normal x: the hardware approximation (rcp.approx.ftz.f64, about
// 2^-22 relative) refined by two Newton steps y += y (1 - x y), each doubling
// the correct bits, to within an ulp: 4 float64 operations where a division
// costs about 7.
__device__ __forceinline__ double rcp64(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = __fma_rn(-x, y, 1.0);
    y = __fma_rn(y, e, y);
    e = __fma_rn(-x, y, 1.0);
    return __fma_rn(y, e, y);
}

// omega / den, 0 when den is 0 (core/level_solver.py:352, 363); subnormal,
// infinite or NaN denominators take the division.  The tests look at the bits
// (integer instructions), not at the value (float64 compares).
__device__ __forceinline__ double omega_over(double omega, double den)
{
    const int hi = __double2hiint(den);
    const int ex = hi & 0x7ff00000;
    if (ex == 0 || ex == 0x7ff00000) {
        if (((hi & 0x7fffffff) | __double2loint(den)) == 0) return 0.0;
        return __ddiv_rn(omega, den);
    }
    return __dmul_rn(omega, rcp64(den));
}

// Coefficients of one pixel for a pass (core/level_solver.py:229-255, 309-364):
// with psi at a tick from the pixel's pass-start du, dv (E in nested fused
// multiply-adds; the reference adds J23 dv twice, hence 2 J23), psi = 1 on the
// first pass, or the stored coefficients of the group's first pass.  On a tick
// W psi = (W a) (E + 1e-5)^(a - 1), with W a and J33 + 1e-5 stored per pixel.
//   A12 = sum_k W psi J12,  BU = lap_u - sum_k W psi J13,  BV = lap_v - sum_k W psi J23,
//   iDu = omega / (wsum + sum_k W psi J11) (0 when the denominator is 0), iDv likewise
//   (omega times the reciprocal: within an ulp or two of the quotient).
// The tensor holds the cross terms doubled (2 J12, 2 J13, 2 J23, exact), as E
// uses them; the sums over them are then twice the sums above, exactly, and
// A12 = sum / 2, BU = fma(-1/2, sum, lap_u) give the same bits.
template <int K, bool CO>
__device__ __forceinline__ Coef64 fold64(const Sor64Args& A, int pk, const FoldIn64<K>& r, double du, double dv)
{
    Coef64 o;
    if (CO && (pk & kPkCoef)) {
        o.A12 = r.j[0];
        o.BU = r.j[1];
        o.BV = r.j[2];
        o.iDu = r.j[3];
        o.iDv = r.j[4];
        return o;
    }
    const bool tick = (pk & kPkTick) != 0;
    double den_u = A.wsum, den_v = A.wsum, a12 = 0.0, c13 = 0.0, c23 = 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double j11 = r.j[0 * K + k], j22 = r.j[1 * K + k], j33 = r.j[2 * K + k];
        const double j12 = r.j[3 * K + k], j13 = r.j[4 * K + k], j23 = r.j[5 * K + k];
        double wp = r.w[k];  // W, or W * a_data on a tick pass
        if (tick) {
            const double a = du, b = dv;
            // E + 1e-5 = a (J11 a + 2 J12 b + 2 J13) + b (J22 b + 2 J23) + (J33 + 1e-5):
            // 5 float64 operations; max(E, 0) + 1e-5 as max(E + 1e-5, 1e-5), compared as
            // 64-bit integers (the order of non-negative doubles; negative ones are below)
            double t = __fma_rn(j11, a, j13);
            t = __fma_rn(j12, b, t);
            const double q = __fma_rn(j22, b, j23);
            double E = __fma_rn(t, a, __fma_rn(q, b, j33));
            if (__double_as_longlong(E) < __double_as_longlong(0.00001)) E = 0.00001;
            wp = __dmul_rn(wp, dpow_b(E, A.a_m1[k], A.pw[k]));
        }
        den_u = __fma_rn(wp, j11, den_u);
        den_v = __fma_rn(wp, j22, den_v);
        a12 = __fma_rn(wp, j12, a12);
        c13 = __fma_rn(wp, j13, c13);
        c23 = __fma_rn(wp, j23, c23);
    }
    o.A12 = __dmul_rn(0.5, a12);
    o.BU = __fma_rn(-0.5, c13, r.lu);
    o.BV = __fma_rn(-0.5, c23, r.lv);
    o.iDu = omega_over(A.omega, den_u);
    o.iDv = omega_over(A.omega, den_v);
    return o;
}

// One SOR update (core/level_solver.py:309-364, a_smooth = 1): c the pixel's
// (du, dv) before it, up/dn the rows above (new) and below (old), lf/rt the
// columns left (new) and right (old), Neumann copies already applied.  du
// first, then dv from the new du; 14 float64 operations.
__device__ __forceinline__ double2 sor_point64(double2 c, double2 up, double2 dn, double2 lf, double2 rt, double2 ca,
                                               double2 cb, double iDv, double wa, double wb, double omm)
{
    double nu = __fma_rn(wa, __dadd_rn(up.x, dn.x), ca.y);
    nu = __fma_rn(wb, __dadd_rn(lf.x, rt.x), nu);
    nu = __fma_rn(-ca.x, c.y, nu);
    const double dun = __fma_rn(nu, cb.y, __dmul_rn(omm, c.x));
    double nv = __fma_rn(wa, __dadd_rn(up.y, dn.y), cb.x);
    nv = __fma_rn(wb, __dadd_rn(lf.y, rt.y), nv);
    nv = __fma_rn(-ca.x, dun, nv);
    const double dvn = __fma_rn(nv, iDv, __dmul_rn(omm, c.y));
    return make_double2(dun, dvn);
}

// Shared memory: CA double2[S][NT] (A12, BU) | CB double2[S][NT] (BV, iDu) |
// CC double[S][NT] (iDv) | X double2[2][NW][2][G] | XE double2[2][2][G].
size_t chain64_smem(int nt)
{
    constexpr int S = 2 * kG64 - 1;
    return (size_t)S * nt * (2 * sizeof(double2) + sizeof(double)) +
           (size_t)(2 * (nt / 32) * 2 * kG64 + 2 * 2 * kG64) * sizeof(double2);
}

// NTM: the most rows (threads) of one CTA, 256, 128 or 64.  The launch bounds
// ask for 1, 3 or 6 CTAs per SM (at most 255 or 170 registers per thread), so
// shorter strips keep 12 warps per SM where 256-row CTAs keep 8.
template <int NT>
struct StripBounds {
    static constexpr int blocks = NT >= 256 ? 1 : (NT >= 128 ? 3 : 6);
};

template <int K, bool CO, bool CL, int NTM>
__global__ void __launch_bounds__(NTM, StripBounds<NTM>::blocks) k_sor_chain64(Sor64Args A, Chain64Table T)
{
    constexpr int G = kG64;
    constexpr int S = 2 * G - 1;
    extern __shared__ __align__(16) double sm64[];
    const DiagGeom g = A.g;
    const int P = g.P, h = g.h, w = g.w;
    const int NT = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, NW = NT >> 5;
    const int nc = CL ? A.nc : 1;
    const int strip = CL ? (int)(blockIdx.x % nc) : 0;
    const int f = CL ? (int)(blockIdx.x / nc) : (int)blockIdx.x;
    const int r = strip * NT + t;  // the level row of this thread
    double2* CA = reinterpret_cast<double2*>(sm64);
    double2* CB = CA + S * NT;
    double* CC = reinterpret_cast<double*>(CB + S * NT);
    double2* X = reinterpret_cast<double2*>(CC + S * NT);
    double2* XE = X + 2 * NW * 2 * G;
    const int pl = g.D * P;
    const double* Jr = A.J + f * A.J_fs + r;
    const double* Wr = A.W + f * A.W_fs + r;
    const double* lapr = A.lap + f * A.lap_fs + r;
    double* coefr = A.coef + f * A.coef_fs + r;
    double* dur = A.du + f * A.st_fs + r;
    double* dvr = A.dv + f * A.st_fs + r;
    double* odu = A.out_du ? A.out_du + f * A.out_fs : nullptr;
    double* odv = A.out_dv ? A.out_dv + f * A.out_fs : nullptr;
    const double omm = A.one_m_omega, wa = A.wa, wb = A.wb;
    const bool row_ok = r < h;
    const bool has_below = r + 1 < h;
    const int last = T.n - 1;
    auto span = [&](int pk) {
        const int G_p = pk >> 8;
        return w + (G_p > 1 ? 2 * (G_p - 1) : 1);
    };

    // pass-start state of the pixel entering at column c of a pass with flags pk,
    // and of the pixel below its left neighbour
    auto fetch_state = [&](int c, int pk, Pre64& p) {
        const bool zero = (pk & kPkZero) != 0;
        const int o = (r + c) * P;
        if (row_ok && c >= 0 && c < w) {
            p.du = zero ? 0.0 : dur[o];
            p.dv = zero ? 0.0 : dvr[o];
        }
        if (has_below && c >= 1 && c <= w) {
            p.nu = zero ? 0.0 : dur[o + 1];
            p.nv = zero ? 0.0 : dvr[o + 1];
        }
    };
    // fold inputs of the pixel at column c of a pass with flags pk
    auto fetch_fold = [&](int c, int pk, FoldIn64<K>& f) {
        const int o = (r + c) * P;
        if (row_ok && c >= 0 && c < w) {
            if (CO && (pk & kPkCoef)) {
#pragma unroll
                for (int q = 0; q < 5; ++q) f.j[q] = coefr[q * pl + o];
            } else {
#pragma unroll
                for (int q = 0; q < 6 * K; ++q) f.j[q] = Jr[q * pl + o];
                const double* wsrc = (pk & kPkTick) ? Wr + K * pl : Wr;  // W * a_data on a tick
#pragma unroll
                for (int k = 0; k < K; ++k) f.w[k] = wsrc[k * pl + o];
                f.lu = lapr[o];
                f.lv = lapr[pl + o];
            }
        }
    };
    auto fold_into = [&](int c, int pk, const FoldIn64<K>& f, const Pre64& p, int slot) {
        if (row_ok && c >= 0 && c < w) {
            const Coef64 cf = fold64<K, CO>(A, pk, f, p.du, p.dv);
            if (CO && (pk & kPkStore)) {
                const int o = (r + c) * P;
                coefr[o] = cf.A12;
                coefr[pl + o] = cf.BU;
                coefr[2 * pl + o] = cf.BV;
                coefr[3 * pl + o] = cf.iDu;
                coefr[4 * pl + o] = cf.iDv;
            }
            CA[slot * NT + t] = make_double2(cf.A12, cf.BU);
            CB[slot * NT + t] = make_double2(cf.BV, cf.iDu);
            CC[slot * NT + t] = cf.iDv;
        }
    };
    auto xs = [&](int par, int wp, int dir, int gi) -> double2& { return X[((par * NW + wp) * 2 + dir) * G + gi]; };
    auto step_barrier = [&]() {
        if constexpr (CL)
            cooperative_groups::this_cluster().sync();
        else
            __syncthreads();
    };
    if constexpr (CL) step_barrier();  // every CTA of the cluster is running before any remote write

    int cp = 0, cstart = 0;
    int pk_cur = T.pk[0];
    int pk_nxt = last > 0 ? T.pk[1] : 0;
    int cend = span(pk_cur);
    Pre64 pre[2];
    fetch_state(-r, pk_cur, pre[0]);
    fetch_state(1 - r, pk_cur, pre[1]);
    {
        FoldIn64<K> f0;
        fetch_fold(-r, pk_cur, f0);
        fold_into(-r, pk_cur, f0, pre[0], 0);
    }
    double2 V0[G], V1[G], V2[G];
#pragma unroll
    for (int gi = 0; gi < G; ++gi) V0[gi] = V1[gi] = V2[gi] = make_double2(0.0, 0.0);

    int total = 0;
    for (int p = 0; p < T.n; ++p) total += span(T.pk[p]);
    const int nsteps = total + h - 1;
    int slot0 = 0;  // s % S
    for (int s0 = 0; s0 < nsteps; s0 += 2) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int s = s0 + q;
            if (s < nsteps) {
                Pre64& cur = pre[q];      // the pixel entering at step s
                Pre64& nxt = pre[q ^ 1];  // the pixel entering at step s + 1
                const int slot1 = slot0 + 1 == S ? 0 : slot0 + 1;
                const int tau = s - r;
                if (tau >= cend && cp < last) {
                    ++cp;
                    cstart = cend;
                    pk_cur = pk_nxt;
                    pk_nxt = cp < last ? T.pk[cp + 1] : 0;
                    cend = cstart + span(pk_cur);
                }
                const bool more = cp < last;
                const bool e_nx = more && tau + 2 >= cend, f_nx = more && tau + 1 >= cend;
                const int Gp = pk_cur >> 8;
                const bool final_out = !more && odu != nullptr;
                const int c0 = tau - cstart;
                const int c_f = f_nx ? tau + 1 - cend : c0 + 1;  // the pixel folded at the end of this step
                const int pk_f = f_nx ? pk_nxt : pk_cur;
                FoldIn64<K> fin;
                fetch_fold(c_f, pk_f, fin);
                const double2 ps0 = make_double2(cur.du, cur.dv);
                const double2 ps1 = make_double2(nxt.du, nxt.dv);
                const double2 dn1 = make_double2(nxt.nu, nxt.nv);
                fetch_state(e_nx ? tau + 2 - cend : c0 + 2, e_nx ? pk_nxt : pk_cur, cur);
                const int pin = (s + 1) & 1;  // parity written at step s - 1
#pragma unroll
                for (int gj = 0; gj < G; ++gj) {
                    const int gi = G - 1 - gj;  // the independent updates first, the newest column last
                    double2 up, dn;
                    up.x = __shfl_up_sync(0xffffffffu, V1[gi].x, 1);
                    up.y = __shfl_up_sync(0xffffffffu, V1[gi].y, 1);
                    if (lane == 0 && warp > 0) up = xs(pin, warp - 1, 0, gi);
                    if (CL && t == 0 && strip > 0) up = XE[(pin * 2 + 0) * G + gi];
                    if (gi == 0) {
                        dn = dn1;
                    } else {
                        dn.x = __shfl_down_sync(0xffffffffu, V1[gi - 1].x, 1);
                        dn.y = __shfl_down_sync(0xffffffffu, V1[gi - 1].y, 1);
                        if (lane == 31 && warp < NW - 1) dn = xs(pin, warp + 1, 1, gi - 1);
                        if (CL && t == NT - 1 && strip < nc - 1) dn = XE[(pin * 2 + 1) * G + gi - 1];
                    }
                    const int c = c0 - 2 * gi;
                    if (gi < Gp && row_ok && c >= 0 && c < w) {
                        const double2 own = gi == 0 ? ps0 : V2[gi - 1];
                        const double2 lf = c > 0 ? V1[gi] : own;
                        const double2 rt = c < w - 1 ? (gi == 0 ? ps1 : V1[gi - 1]) : own;
                        const double2 u_ = r > 0 ? up : own;
                        const double2 d_ = r < h - 1 ? dn : own;
                        int sl = slot0 - 2 * gi;
                        if (sl < 0) sl += S;
                        V0[gi] = sor_point64(own, u_, d_, lf, rt, CA[sl * NT + t], CB[sl * NT + t], CC[sl * NT + t],
                                             wa, wb, omm);
                        if (gi == Gp - 1) {
                            if (final_out) {
                                odu[(long long)r * A.out_rs + c] = V0[gi].x;
                                odv[(long long)r * A.out_rs + c] = V0[gi].y;
                            } else {
                                dur[(r + c) * P] = V0[gi].x;
                                dvr[(r + c) * P] = V0[gi].y;
                            }
                        }
                    }
                }
                fold_into(c_f, pk_f, fin, nxt, slot1);
                const int pout = s & 1;
                if (lane == 31) {
#pragma unroll
                    for (int gi = 0; gi < G; ++gi) xs(pout, warp, 0, gi) = V0[gi];
                }
                if (lane == 0) {
#pragma unroll
                    for (int gi = 0; gi + 1 < G; ++gi) xs(pout, warp, 1, gi) = V0[gi];
                }
                if constexpr (CL) {
                    if (t == NT - 1 && strip < nc - 1) {
                        double2* dst = cooperative_groups::this_cluster().map_shared_rank(XE, strip + 1);
#pragma unroll
                        for (int gi = 0; gi < G; ++gi) dst[(pout * 2 + 0) * G + gi] = V0[gi];
                    }
                    if (t == 0 && strip > 0) {
                        double2* dst = cooperative_groups::this_cluster().map_shared_rank(XE, strip - 1);
#pragma unroll
                        for (int gi = 0; gi + 1 < G; ++gi) dst[(pout * 2 + 1) * G + gi] = V0[gi];
                    }
                }
#pragma unroll
                for (int gi = 0; gi < G; ++gi) {
                    V2[gi] = V1[gi];
                    V1[gi] = V0[gi];
                }
                slot0 = slot1;
            }
            step_barrier();
        }
    }
}

// Row strips of a level with at most `rows` rows per CTA (256, 128 or 64): one
// CTA when the level fits, else nc CTAs of nt rows (a cluster when nc > 1).
void split64(const DiagGeom& g, int rows, int* nc, int* nt)
{
    const int n = (g.P + rows - 1) / rows;
    *nc = n;
    *nt = ((g.P + n - 1) / n + 31) / 32 * 32;
}

template <int K, bool CO, bool CL, int NTM>
cudaError_t run_chain64_t(const Sor64Args& A, const Chain64Table& T, int n_frames, int nt, cudaStream_t st)
{
    const size_t smem = chain64_smem(nt);
    const cudaError_t e = ensure_max_dyn_smem((const void*)k_sor_chain64<K, CO, CL, NTM>, kSmem64);
    if (e != cudaSuccess) return e;
    if constexpr (!CL) {
        k_sor_chain64<K, CO, false, NTM><<<n_frames, nt, smem, st>>>(A, T);
        return cudaGetLastError();
    } else {
        if (A.nc > kPortableStrips) {
            const cudaError_t e2 = ensure_nonportable_clusters((const void*)k_sor_chain64<K, CO, true, NTM>);
            if (e2 != cudaSuccess) return e2;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(n_frames * A.nc));
        cfg.blockDim = dim3((unsigned)nt);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)A.nc;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_sor_chain64<K, CO, true, NTM>, A, T);
    }
}

template <int K, int NTM>
cudaError_t run_chain64_n(const Sor64Args& A, const Chain64Table& T, bool co, int n_frames, int nt, cudaStream_t st)
{
    if (A.nc == 1)
        return co ? run_chain64_t<K, true, false, NTM>(A, T, n_frames, nt, st)
                  : run_chain64_t<K, false, false, NTM>(A, T, n_frames, nt, st);
    return co ? run_chain64_t<K, true, true, NTM>(A, T, n_frames, nt, st)
              : run_chain64_t<K, false, true, NTM>(A, T, n_frames, nt, st);
}

template <int K>
cudaError_t run_chain64(const Sor64Args& A, const Chain64Table& T, bool co, int n_frames, int nt, cudaStream_t st)
{
    if (nt <= 64) return run_chain64_n<K, 64>(A, T, co, n_frames, nt, st);
    if (nt <= 128) return run_chain64_n<K, 128>(A, T, co, n_frames, nt, st);
    return run_chain64_n<K, 256>(A, T, co, n_frames, nt, st);
}

}  // namespace

bool sor_chain64_rows_ok(const DiagGeom& g, int rows)
{
    if (rows != 64 && rows != 128 && rows != kLane64) return false;
    int nc, nt;
    split64(g, rows, &nc, &nt);
    return nc <= kMaxStrips64 && chain64_smem(nt) <= (size_t)kSmem64;
}

int sor_chain64_default_rows(const DiagGeom& g, int n_frames, int n_sms)
{
    // levels over 512 rows: 128-row strips (three CTAs per SM) while the cluster
    // stays within 16 CTAs
    if (g.P > 512 && sor_chain64_rows_ok(g, 128)) return 128;
    // the tallest strips that still give every SM work; shorter strips where a
    // batch of few frames would leave SMs idle (one frame per call: 8 strips)
    for (int rows = kLane64; rows >= 64; rows /= 2) {
        if (!sor_chain64_rows_ok(g, rows)) break;
        const long long ctas = (long long)n_frames * ((g.P + rows - 1) / rows);
        if (ctas >= n_sms) return rows;
    }
    for (int rows = 64; rows <= kLane64; rows *= 2)
        if (sor_chain64_rows_ok(g, rows)) return rows;
    return kLane64;
}

bool sor_chain64_supports(int K, const DiagGeom& g, int n_passes)
{
    if (K < 1 || K > 4 || (g.P & 31) || g.w < 3 || n_passes < 1 || n_passes > kMaxChain) return false;
    int nc, nt;
    split64(g, kLane64, &nc, &nt);
    // 32-bit offsets within a frame: the largest plane index read is (6K + 2) planes of D * P
    const long long plane = (long long)g.D * g.P;
    // the tallest strips must fit a portable cluster: the fallback of a refused larger cluster
    return nc <= kPortableStrips && plane * (6 * K + 2) < 0x7fffffffLL && chain64_smem(nt) <= (size_t)kSmem64;
}

cudaError_t launch_sor_chain64(const double* J, long long J_fs, const double* W, long long W_fs, const double* lap,
                               long long lap_fs, double* coef, long long coef_fs, double* du, double* dv,
                               long long st_fs, int n_frames, int K, DiagGeom g, const ChainPass* passes,
                               int n_passes, const double* a_data, double wx, double wy, double omega,
                               cudaStream_t st, double* out_du, double* out_dv, long long out_fs, int out_rs,
                               int rows, const PowTab64* pows)
{
    if (!sor_chain64_supports(K, g, n_passes) || n_frames < 1) return cudaErrorInvalidValue;
    if (rows == 0) rows = kLane64;
    if (!sor_chain64_rows_ok(g, rows)) return cudaErrorInvalidValue;
    int nc = 0, nt = 0;
    split64(g, rows, &nc, &nt);
    if ((long long)n_frames * nc > 0x7fffffffLL) return cudaErrorInvalidValue;
    Chain64Table T;
    T.n = n_passes;
    bool co = false;
    for (int p = 0; p < n_passes; ++p) {
        const ChainPass& q = passes[p];
        if (q.G < 1 || q.G > kG64 || q.mode < -1 || q.mode > 3) return cudaErrorInvalidValue;
        const bool coef_in = q.mode < 0, store = q.mode >= 0 && q.store_coef;
        T.pk[p] = (q.G << 8) | (store ? kPkStore : 0) | (coef_in ? kPkCoef : 0) |
                  (!coef_in && (q.mode & 2) ? kPkTick : 0) | (!coef_in && (q.mode & 1) ? kPkZero : 0);
        co = co || coef_in || store;
    }
    for (int p = n_passes; p < kMaxChain; ++p) T.pk[p] = 1 << 8;
    Sor64Args A;
    A.J = J;
    A.J_fs = J_fs;
    A.W = W;
    A.W_fs = W_fs;
    A.lap = lap;
    A.lap_fs = lap_fs;
    A.coef = coef;
    A.coef_fs = coef_fs;
    A.du = du;
    A.dv = dv;
    A.st_fs = st_fs;
    A.out_du = out_du;
    A.out_dv = out_dv;
    A.out_fs = out_fs;
    A.out_rs = out_rs;
    A.g = g;
    A.wa = wy;  // the thread index runs along rows: row neighbours carry the y weight
    A.wb = wx;
    A.wsum = ((wx + wx) + wy) + wy;
    A.omega = omega;
    A.one_m_omega = 1.0 - omega;
    for (int k = 0; k < kMaxK; ++k) {
        A.a_m1[k] = k < K ? a_data[k] - 1.0 : 0.0;
        A.pw[k] = pows && k < K ? pows[k] : PowTab64();
    }
    auto launch = [&](int nc_, int nt_) {
        A.nc = nc_;
        switch (K) {
            case 1: return run_chain64<1>(A, T, co, n_frames, nt_, st);
            case 2: return run_chain64<2>(A, T, co, n_frames, nt_, st);
            case 3: return run_chain64<3>(A, T, co, n_frames, nt_, st);
            default: return run_chain64<4>(A, T, co, n_frames, nt_, st);
        }
    };
    cudaError_t e = launch(nc, nt);
    if (e != cudaSuccess && nc > kPortableStrips) {
        // a device that cannot schedule a cluster this large refuses the launch (nothing ran, the
        // error is not sticky): the tallest strips give the same bits with at most 8 CTAs
        cudaGetLastError();
        split64(g, kLane64, &nc, &nt);
        e = launch(nc, nt);
    }
    return e;
}

}  // namespace frg
