// Exact-order wavefront SOR with the coefficient fold in its diagonal loader.
//
// Same schedule as k_sor (pixel (r, c) of pass iteration g at step r + c + 2g,
// one __syncthreads per step; core/level_solver.py:257-364 order), with three
// changes:
//  * the loader builds the five per-pixel coefficients itself from J, W, lap
//    and (at a psi tick) the pixel's du, dv (core/level_solver.py:229-255,
//    342-364), so no separate fold pass reads and writes them through HBM;
//  * the work of a step -- every pixel of the active diagonals -- is spread
//    evenly over all threads instead of one row per thread, so threads whose
//    row misses the active diagonals no longer idle while others carry G
//    updates;
//  * ring slots hold (du, dv) as float2 and the coefficients as float4 + float,
//    so an update issues 7 shared-memory loads instead of 15.
// Ring slot (7P floats): [du,dv] float2[P] | [A12, BU, BV, 1/den_u] float4[P] | 1/den_v float[P].
// The ring has 2G+3 slots: the diagonal written back at step s (s - 2G) and the
// one stored at step s (s + 2) never share a slot, because a different thread
// handles a given row in the two operations.
#include "frg_internal.h"

#include <cooperative_groups.h>

namespace frg {

namespace {

struct SorArgs {
    const float* J;      // [6][K][D*P] per frame
    long long J_fs;
    const float* W;      // [K][D*P] per frame (W_fs 0: shared)
    long long W_fs;
    const float* lap;    // [2][D*P]
    long long lap_fs;
    float* coef;         // [5][D*P], read when mode < 0, written when store_coef
    long long coef_fs;
    float* du;
    float* dv;
    long long st_fs;
    float* out_du;       // when set, this pass writes du, dv row-major (h, w) here instead
    float* out_dv;
    long long out_fs;
    DiagGeom g;
    int G;
    int mode;            // -1: coefficients from `coef`; else bit0 du=dv=0, bit1 psi tick
    int store_coef;
    float wa, wb;        // smoothness weights along the lane (rows) and across it
    float wsum;          // 2 wx + 2 wy, summed as the reference does
    float omega;
    float a_data[kMaxK];
    int nc;              // k_sor_regs cluster form: CTAs (row strips) per frame
};

__device__ __forceinline__ int rmin_of(const DiagGeom& g, int d) { return d - (g.w - 1) > 0 ? d - (g.w - 1) : 0; }
__device__ __forceinline__ int rmax_of(const DiagGeom& g, int d) { return d < g.h - 1 ? d : g.h - 1; }

// raw inputs of one pixel of a diagonal
template <int K>
struct Raw {
    float j[6 * K];
    float w[K];
    float lu, lv, du, dv;
};

template <int K>
__device__ __forceinline__ void load_raw(const SorArgs& A, const float* J, const float* W, const float* lap,
                                         const float* coef, const float* du, const float* dv, long long o,
                                         long long plane, Raw<K>& r)
{
    if (A.mode < 0) {
#pragma unroll
        for (int q = 0; q < 5; ++q) r.j[q] = coef[q * plane + o];
    } else {
#pragma unroll
        for (int q = 0; q < 6; ++q)
#pragma unroll
            for (int k = 0; k < K; ++k) r.j[q * K + k] = J[((long long)q * K + k) * plane + o];
#pragma unroll
        for (int k = 0; k < K; ++k) r.w[k] = W[(long long)k * plane + o];
        r.lu = lap[o];
        r.lv = lap[plane + o];
    }
    if (A.mode >= 0 && (A.mode & 1)) {
        r.du = 0.0f;
        r.dv = 0.0f;
    } else {
        r.du = du[o];
        r.dv = dv[o];
    }
}

// The five coefficients of one pixel: stored ones passed through (mode < 0),
// or folded from J, W, lap and, at a psi tick, the pixel's du, dv
// (core/level_solver.py:229-255, 342-364).  Explicit round-to-nearest
// intrinsics fix every rounding, so every kernel that folds through here
// gets the same bits.
struct Coef {
    float A12, BU, BV, iDu, iDv;
};

template <int K>
__device__ __forceinline__ Coef fold_m(const SorArgs& A, int mode, const Raw<K>& r)
{
    Coef o;
    if (mode < 0) {
        o.A12 = r.j[0];
        o.BU = r.j[1];
        o.BV = r.j[2];
        o.iDu = r.j[3];
        o.iDv = r.j[4];
        return o;
    }
    const bool tick = (mode & 2) != 0;
    float A11 = 0.f, A22 = 0.f, a12 = 0.f, C13 = 0.f, C23 = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float j11 = r.j[0 * K + k], j22 = r.j[1 * K + k], j33 = r.j[2 * K + k];
        const float j12 = r.j[3 * K + k], j13 = r.j[4 * K + k], j23 = r.j[5 * K + k];
        float psi = 1.0f;
        if (tick) {
            const float a = r.du, b = r.dv;
            // E = J11 a a + J22 b b + 2 J23 b + 2 J12 a b + 2 J13 a + J33 (the reference adds J23 b
            // twice) as a chain of fused multiply-adds: E cancels to near zero where the
            // linearisation fits, and each fused step rounds once
            float E = __fmaf_rn(__fmul_rn(2.0f, j13), a, j33);
            E = __fmaf_rn(__fmul_rn(2.0f, j23), b, E);
            E = __fmaf_rn(__fmul_rn(__fmul_rn(2.0f, j12), a), b, E);
            E = __fmaf_rn(__fmul_rn(j22, b), b, E);
            E = __fmaf_rn(__fmul_rn(j11, a), a, E);
            E = fmaxf(E, 0.0f);
            // (E + eps)^(a_k - 1) as exp2((a_k - 1) log2(E + eps)) on the special-function
            // unit: relative error ~1e-6, the fp32 path's rounding level
            psi = __fmul_rn(A.a_data[k],
                            exp2f(__fmul_rn(__fsub_rn(A.a_data[k], 1.0f), __log2f(__fadd_rn(E, 1e-5f)))));
        }
        const float wp = __fmul_rn(r.w[k], psi);
        A11 = __fmaf_rn(wp, j11, A11);
        A22 = __fmaf_rn(wp, j22, A22);
        a12 = __fmaf_rn(wp, j12, a12);
        C13 = __fmaf_rn(wp, j13, C13);
        C23 = __fmaf_rn(wp, j23, C23);
    }
    const float den_u = __fadd_rn(A.wsum, A11), den_v = __fadd_rn(A.wsum, A22);
    o.A12 = a12;
    o.BU = __fsub_rn(r.lu, C13);
    o.BV = __fsub_rn(r.lv, C23);
    o.iDu = den_u != 0.0f ? __frcp_rn(den_u) : 0.0f;
    o.iDv = den_v != 0.0f ? __frcp_rn(den_v) : 0.0f;
    return o;
}

template <int K>
__device__ __forceinline__ Coef fold(const SorArgs& A, const Raw<K>& r)
{
    return fold_m<K>(A, A.mode, r);
}

__device__ __forceinline__ void store_coef(const SorArgs& A, const Coef& c, float* coef, long long o, long long plane)
{
    if (A.mode >= 0 && A.store_coef) {
        coef[o] = c.A12;
        coef[plane + o] = c.BU;
        coef[2 * plane + o] = c.BV;
        coef[3 * plane + o] = c.iDu;
        coef[4 * plane + o] = c.iDv;
    }
}

// fold (or pass the stored coefficients through) and store into ring row a
template <int K>
__device__ __forceinline__ void put_raw(const SorArgs& A, const Raw<K>& r, float2* DV, float4* C4, float* C1, int a,
                                        float* coef, long long o, long long plane)
{
    const Coef c = fold<K>(A, r);
    store_coef(A, c, coef, o, plane);
    DV[a] = make_float2(r.du, r.dv);
    C4[a] = make_float4(c.A12, c.BU, c.BV, c.iDu);
    C1[a] = c.iDv;
}

// One SOR update of a pixel (core/level_solver.py:309-364 with a_smooth = 1):
// c its (du, dv) before the update; up/dn the row above (new) and below (old),
// lf/rt the column left (new) and right (old), Neumann copies already applied;
// wa weights the row neighbours, wb the column neighbours.  du first, then dv
// from the new du.
__device__ __forceinline__ float2 sor_point(float2 c, float2 up, float2 dn, float2 lf, float2 rt, float4 c4, float iDv,
                                            float wa, float wb, float omega, float one_m_omega)
{
    float nu = __fmaf_rn(wa, __fadd_rn(up.x, dn.x), __fmul_rn(wb, __fadd_rn(lf.x, rt.x)));
    nu = __fadd_rn(nu, c4.y);
    nu = __fmaf_rn(-c4.x, c.y, nu);
    const float dun = __fmaf_rn(one_m_omega, c.x, __fmul_rn(omega, __fmul_rn(nu, c4.w)));
    float nv = __fmaf_rn(wa, __fadd_rn(up.y, dn.y), __fmul_rn(wb, __fadd_rn(lf.y, rt.y)));
    nv = __fadd_rn(nv, c4.z);
    nv = __fmaf_rn(-c4.x, dun, nv);
    const float dvn = __fmaf_rn(one_m_omega, c.y, __fmul_rn(omega, __fmul_rn(nv, iDv)));
    return make_float2(dun, dvn);
}

template <int K, int PF, int MAXT>
__global__ void __launch_bounds__(MAXT) k_sor_fused(SorArgs A)
{
    extern __shared__ __align__(16) float sm[];
    const DiagGeom g = A.g;
    const int P = g.P, D = g.D, Hh = g.h, Bw = g.w, G = A.G;
    const int R = 2 * G + 3;
    const int tid = threadIdx.x, nth = blockDim.x;
    const long long plane = (long long)D * P;
    const int f = blockIdx.x;
    const float* J = A.J + f * A.J_fs;
    const float* W = A.W + f * A.W_fs;
    const float* lap = A.lap + f * A.lap_fs;
    float* coef = A.coef + f * A.coef_fs;
    float* du = A.du + f * A.st_fs;
    float* dv = A.dv + f * A.st_fs;
    const float omega = A.omega, one_m_omega = 1.0f - omega, wa = A.wa, wb = A.wb;

    auto slot_dv = [&](int slot) { return reinterpret_cast<float2*>(sm + (long long)slot * 7 * P); };
    auto slot_c4 = [&](int slot) { return reinterpret_cast<float4*>(sm + (long long)slot * 7 * P + 2 * P); };
    auto slot_c1 = [&](int slot) { return sm + (long long)slot * 7 * P + 6 * P; };

    // loader: thread t takes row rmin(d) + t of diagonal d (coalesced)
    Raw<K> buf[PF];
    auto fetch = [&](int d, Raw<K>& r) {
        if (d >= 0 && d < D) {
            const int a = rmin_of(g, d) + tid;
            if (a <= rmax_of(g, d)) load_raw<K>(A, J, W, lap, coef, du, dv, (long long)d * P + a, plane, r);
        }
    };
    auto store = [&](int d, int sl, const Raw<K>& r) {
        if (d >= 0 && d < D) {
            const int a = rmin_of(g, d) + tid;
            if (a <= rmax_of(g, d))
                put_raw<K>(A, r, slot_dv(sl), slot_c4(sl), slot_c1(sl), a, coef, (long long)d * P + a, plane);
        }
    };
    float* odu = A.out_du ? A.out_du + f * A.out_fs : nullptr;
    float* odv = A.out_dv ? A.out_dv + f * A.out_fs : nullptr;
    auto writeback = [&](int d, int sl) {
        if (d >= 0 && d < D) {
            const int a = rmin_of(g, d) + tid;
            if (a <= rmax_of(g, d)) {
                const float2 v = slot_dv(sl)[a];
                if (odu) {
                    // row-major for the median; the strided sectors of one step
                    // are completed by the following steps while still in L2
                    const long long o = (long long)a * Bw + (d - a);
                    odu[o] = v.x;
                    odv[o] = v.y;
                } else {
                    du[(long long)d * P + a] = v.x;
                    dv[(long long)d * P + a] = v.y;
                }
            }
        }
    };

    {
        Raw<K> r0, r1;
        fetch(0, r0);
        fetch(1, r1);
        store(0, 0, r0);
        store(1, 1, r1);
    }
#pragma unroll
    for (int j = 0; j < PF; ++j) fetch(2 + j, buf[(2 + j) % PF]);
    __syncthreads();

    const int nsteps = D + 2 * (G - 1);
    int slot_s = 0;  // s % R, advanced once per step
    for (int s0 = 0; s0 < nsteps; s0 += PF) {
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            const int s = s0 + q;
            if (s < nsteps) {
                // Ring maintenance first, so the fold's latency overlaps the
                // updates below: diagonal s - 2G leaves (last read at step
                // s - 1), diagonal s + 2 enters (first read at step s + 1); no
                // update of this step touches either slot.  With R = 2G + 3,
                // s - 2G and s + 3 share a slot.
                int sl_out = slot_s + 3, sl_in = slot_s + 2;
                if (sl_out >= R) sl_out -= R;
                if (sl_in >= R) sl_in -= R;
                writeback(s - 2 * G, sl_out);
                store(s + 2, sl_in, buf[(q + 2) % PF]);
                fetch(s + 2 + PF, buf[(q + 2) % PF]);
                // Active diagonals d = s - 2*gi.  Their pixels, concatenated in gi
                // order, are dealt round-robin to the threads: thread t takes, on
                // diagonal gi, the row at offset (t - prefix_gi) mod nth, which
                // is at most one row since no diagonal is longer than nth.
                int pmod = 0;  // prefix of the pixel list, modulo nth (len <= nth)
#pragma unroll
                for (int gi = 0; gi < kGMax; ++gi) {
                    const int d = s - 2 * gi;
                    if (gi >= G || d < 0) break;
                    if (d >= D) continue;
                    const int r0 = rmin_of(g, d);
                    const int len = rmax_of(g, d) - r0 + 1;
                    int off = tid - pmod;
                    if (off < 0) off += nth;
                    pmod += len;
                    if (pmod >= nth) pmod -= nth;
                    if (off >= len) continue;
                    const int a = r0 + off;
                    const int b = d - a;
                    int sl = slot_s - 2 * gi;
                    if (sl < 0) sl += R;
                    const int slm = sl == 0 ? R - 1 : sl - 1;
                    const int slp = sl == R - 1 ? 0 : sl + 1;
                    float2* DVc = slot_dv(sl);
                    const float2* DVm = slot_dv(slm);
                    const float2* DVp = slot_dv(slp);
                    const float2 c = DVc[a];
                    const float4 c4 = slot_c4(sl)[a];
                    const float iDv = slot_c1(sl)[a];
                    const float2 am = a > 0 ? DVm[a - 1] : c;
                    const float2 bm = b > 0 ? DVm[a] : c;
                    const float2 ap = a < Hh - 1 ? DVp[a + 1] : c;
                    const float2 bp = b < Bw - 1 ? DVp[a] : c;
                    DVc[a] = sor_point(c, am, ap, bm, bp, c4, iDv, wa, wb, omega, one_m_omega);
                }
                if (++slot_s == R) slot_s = 0;
            }
            __syncthreads();
        }
    }
    for (int e = nsteps - 2 * G > 0 ? nsteps - 2 * G : 0; e < D; ++e) writeback(e, e % R);
}

// ---------------------------------------------------------------------------
// The same exact-order SOR pass with one thread per row and the state in
// registers.  Thread r updates, at step s, pixel (r, s - r - 2 gi) of every
// pipelined iteration gi (the schedule above).  Every neighbour the update
// reads was produced one step earlier, so it travels without shared memory:
//   left  (r, c - 1), iteration gi      this thread, step s - 1, iteration gi
//   right (r, c + 1), iteration gi - 1  this thread, step s - 1, iteration gi - 1
//   own   (r, c),     iteration gi - 1  this thread, step s - 2, iteration gi - 1
//   up    (r - 1, c), iteration gi      thread r - 1, step s - 1, iteration gi (shfl_up)
//   down  (r + 1, c), iteration gi - 1  thread r + 1, step s - 1, iteration gi - 1 (shfl_down)
// Iteration gi = 0 reads the pass-start state in place of "iteration -1":
// the thread's own pixels on diagonals s and s + 1 and row r + 1's pixel on
// diagonal s + 1, all loaded two steps ahead with the raw fold inputs of the
// entering pixel (r, s - r).  Lanes 0 and 31 take the cross-warp neighbours
// from a two-parity exchange buffer written in the previous step; one
// __syncthreads per step.  A pixel's coefficients, folded when it enters, stay
// in a per-thread ring of 2G - 1 shared-memory slots until its last update.
// Shared memory: C4 float4[S][NT] | C1 float[S][NT] | X float2[2][NW][2][G]
// | XE float2[2][2][G].
//
// Cluster form (CL): levels taller than one CTA split their rows into nc
// strips of NT rows, one CTA per strip, the nc CTAs of a frame forming a
// thread-block cluster.  The strips' edge rows exchange their values through
// distributed shared memory (each writes into the neighbouring CTA's XE) and a
// cluster barrier replaces __syncthreads, so the strips advance step by step
// as one wavefront.
// ---------------------------------------------------------------------------
template <int K>
struct Pre {
    Raw<K> raw;   // pixel (r, d - r)
    float nu, nv; // pass-start du, dv of pixel (r + 1, d - r - 1)
};

template <int K, int G, bool CL>
__global__ void __launch_bounds__(kMaxLane) k_sor_regs(SorArgs A)
{
    extern __shared__ __align__(16) float sm[];
    constexpr int S = 2 * G - 1;
    const DiagGeom g = A.g;
    const int P = g.P, D = g.D, h = g.h, w = g.w;
    const int NT = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, NW = NT >> 5;
    const int nc = CL ? A.nc : 1;
    const int strip = CL ? (int)(blockIdx.x % nc) : 0;
    const int f = CL ? (int)(blockIdx.x / nc) : (int)blockIdx.x;
    const int r = strip * NT + t;  // the level row of this thread
    float4* C4 = reinterpret_cast<float4*>(sm);
    float* C1 = sm + 4 * S * NT;
    float2* X = reinterpret_cast<float2*>(C1 + S * NT);
    float2* XE = X + 2 * NW * 2 * G;  // [par][0: row above the strip, 1: row below][gi]
    const long long plane = (long long)D * P;
    const float* J = A.J + f * A.J_fs;
    const float* W = A.W + f * A.W_fs;
    const float* lap = A.lap + f * A.lap_fs;
    float* coef = A.coef + f * A.coef_fs;
    float* du = A.du + f * A.st_fs;
    float* dv = A.dv + f * A.st_fs;
    float* odu = A.out_du ? A.out_du + f * A.out_fs : nullptr;
    float* odv = A.out_dv ? A.out_dv + f * A.out_fs : nullptr;
    const float omega = A.omega, one_m_omega = 1.0f - omega, wa = A.wa, wb = A.wb;
    const bool zero_start = A.mode >= 0 && (A.mode & 1);
    const bool row_ok = r < h;
    const bool has_below = r + 1 < h;

    auto fetch = [&](int d, Pre<K>& p) {
        const int c = d - r;
        if (row_ok && c >= 0 && c < w) load_raw<K>(A, J, W, lap, coef, du, dv, (long long)d * P + r, plane, p.raw);
        if (has_below && c >= 1 && c <= w) {
            if (zero_start) {
                p.nu = 0.0f;
                p.nv = 0.0f;
            } else {
                p.nu = du[(long long)d * P + r + 1];
                p.nv = dv[(long long)d * P + r + 1];
            }
        }
    };
    // exchange slot: parity, warp, direction (0: this warp's lane 31 for the warp below,
    // 1: lane 0 for the warp above), iteration
    auto xs = [&](int par, int wp, int dir, int gi) -> float2& { return X[((par * NW + wp) * 2 + dir) * G + gi]; };
    auto step_barrier = [&]() {
        if constexpr (CL)
            cooperative_groups::this_cluster().sync();
        else
            __syncthreads();
    };
    if constexpr (CL) step_barrier();  // every CTA of the cluster is running before any remote write

    Pre<K> pre[2];
    fetch(0, pre[0]);
    fetch(1, pre[1]);
    float2 V0[G], V1[G], V2[G];
#pragma unroll
    for (int gi = 0; gi < G; ++gi) V0[gi] = V1[gi] = V2[gi] = make_float2(0.0f, 0.0f);

    const int nsteps = D + 2 * (G - 1);
    int slot0 = 0;  // s % S
    for (int s0 = 0; s0 < nsteps; s0 += 2) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int s = s0 + q;
            if (s < nsteps) {
                Pre<K>& cur = pre[q];       // diagonal s
                Pre<K>& nxt = pre[q ^ 1];   // diagonal s + 1
                const int c0 = s - r;
                const float2 ps0 = make_float2(cur.raw.du, cur.raw.dv);
                const float2 ps1 = make_float2(nxt.raw.du, nxt.raw.dv);
                const float2 dn1 = make_float2(nxt.nu, nxt.nv);
                if (row_ok && c0 >= 0 && c0 < w) {
                    const Coef cf = fold<K>(A, cur.raw);
                    store_coef(A, cf, coef, (long long)s * P + r, plane);
                    C4[slot0 * NT + t] = make_float4(cf.A12, cf.BU, cf.BV, cf.iDu);
                    C1[slot0 * NT + t] = cf.iDv;
                }
                fetch(s + 2, cur);
                const int pin = (s + 1) & 1;  // parity written at step s - 1
#pragma unroll
                for (int gi = 0; gi < G; ++gi) {
                    float2 up, dn;
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
                    if (row_ok && c >= 0 && c < w) {
                        const float2 own = gi == 0 ? ps0 : V2[gi - 1];
                        const float2 lf = c > 0 ? V1[gi] : own;
                        const float2 rt = c < w - 1 ? (gi == 0 ? ps1 : V1[gi - 1]) : own;
                        const float2 u_ = r > 0 ? up : own;
                        const float2 d_ = r < h - 1 ? dn : own;
                        int sl = slot0 - 2 * gi;
                        if (sl < 0) sl += S;
                        V0[gi] = sor_point(own, u_, d_, lf, rt, C4[sl * NT + t], C1[sl * NT + t], wa, wb, omega,
                                           one_m_omega);
                        if (gi == G - 1) {
                            if (odu) {
                                const long long o = (long long)r * w + c;
                                odu[o] = V0[gi].x;
                                odv[o] = V0[gi].y;
                            } else {
                                const long long o = (long long)(r + c) * P + r;
                                du[o] = V0[gi].x;
                                dv[o] = V0[gi].y;
                            }
                        }
                    }
                }
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
                    // strip edges: the last row feeds the next strip's "up", the first row the
                    // previous strip's "down", in the neighbouring CTA's shared memory
                    if (t == NT - 1 && strip < nc - 1) {
                        float2* dst = cooperative_groups::this_cluster().map_shared_rank(XE, strip + 1);
#pragma unroll
                        for (int gi = 0; gi < G; ++gi) dst[(pout * 2 + 0) * G + gi] = V0[gi];
                    }
                    if (t == 0 && strip > 0) {
                        float2* dst = cooperative_groups::this_cluster().map_shared_rank(XE, strip - 1);
#pragma unroll
                        for (int gi = 0; gi + 1 < G; ++gi) dst[(pout * 2 + 1) * G + gi] = V0[gi];
                    }
                }
#pragma unroll
                for (int gi = 0; gi < G; ++gi) {
                    V2[gi] = V1[gi];
                    V1[gi] = V0[gi];
                }
                if (++slot0 == S) slot0 = 0;
            }
            step_barrier();
        }
    }
}

// ---------------------------------------------------------------------------
// k_sor_chain: every pass of a level in one launch of the rows-in-registers
// schedule.  A row's local time is tau = s - r; pass p occupies the local
// times [start_p, start_p + span_p) with span_p = w + 2(G_p - 1) (w + 1 for
// G_p = 1: the prefetch at column w of a pass loads the pass-start value below
// the pass's last column), and pass p + 1 starts where pass p ends, so a row
// goes from its last update of one pass to its first of the next without
// waiting for the wavefront to drain and refill.  Within a pass
// everything is as in k_sor_regs (pixel (r, c), iteration gi at tau =
// start_p + c + 2 gi).  The passes never overlap in one row (pass p's last
// column c = w - 1 of its last iteration falls before pass p + 1's column 0),
// so the per-row register state serves them one after the other.  Between
// passes the state goes through du, dv in global memory as between launches:
// a row's final value of pass p at (r, c) is stored at tau = start_p + c +
// 2(G_p - 1) and read back for pass p + 1 at least w - 2 steps later (the
// row below's value too, so past at least one barrier for w >= 3).
// Each row keeps one cursor, the pass of its updates (tau), with the flags of
// that pass and the next; the coefficient fold (tau + 1: the fold of the
// diagonal entering next step runs after this step's updates, off their
// critical path) and the prefetch (tau + 2) fall in the one or the other,
// since every span is at least 4.  The ring slot of a pixel is its entry step
// mod (2G - 1), as in k_sor_regs.
// Offsets within a frame are 32-bit (the host checks the plane sizes).
// ---------------------------------------------------------------------------
// Pass table: one packed word per pass, G << 8 | store << 3 | coef << 2 |
// tick << 1 | zero (zero: du = dv = 0 at the pass start; tick: psi from the
// pass-start du, dv; coef: the folded coefficients are read back instead of
// folded; store: the fold also writes them for the passes that read them).
struct ChainTable {
    int n;
    int pk[kMaxChain];
};

constexpr int kPkZero = 1, kPkTick = 2, kPkCoef = 4, kPkStore = 8;

// fold of k_sor_regs (fold_m) with the pass's mode given as flags
template <int K, bool CO>
__device__ __forceinline__ Coef fold_pk(const SorArgs& A, int pk, const Raw<K>& r)
{
    if (CO && (pk & kPkCoef)) return fold_m<K>(A, -1, r);
    return fold_m<K>(A, (pk & kPkTick) ? 2 : 0, r);
}

// CL: the level's rows are cut into A.nc strips of NT rows, one CTA each, the
// strips of a frame forming a thread-block cluster, exactly as k_sor_regs's
// cluster form (edge rows through distributed shared memory, a cluster barrier
// per step; every CTA runs the same step count).
template <int K, int G, bool CO, bool CL>
__global__ void __launch_bounds__(kMaxLane) k_sor_chain(SorArgs A, ChainTable T)
{
    extern __shared__ __align__(16) float sm[];
    constexpr int S = 2 * G - 1;
    const DiagGeom g = A.g;
    const int P = g.P, h = g.h, w = g.w;
    const int NT = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, NW = NT >> 5;
    const int nc = CL ? A.nc : 1;
    const int strip = CL ? (int)(blockIdx.x % nc) : 0;
    const int f = CL ? (int)(blockIdx.x / nc) : (int)blockIdx.x;
    const int r = strip * NT + t;  // the level row of this thread
    float4* C4 = reinterpret_cast<float4*>(sm);
    float* C1 = sm + 4 * S * NT;
    float2* X = reinterpret_cast<float2*>(C1 + S * NT);
    float2* XE = X + 2 * NW * 2 * G;  // [par][0: row above the strip, 1: row below][gi]
    const int pl = g.D * P;
    const float* Jr = A.J + f * A.J_fs + r;
    const float* Wr = A.W + f * A.W_fs + r;
    const float* lapr = A.lap + f * A.lap_fs + r;
    float* coefr = A.coef + f * A.coef_fs + r;
    float* dur = A.du + f * A.st_fs + r;
    float* dvr = A.dv + f * A.st_fs + r;
    float* odu = A.out_du ? A.out_du + f * A.out_fs : nullptr;
    float* odv = A.out_dv ? A.out_dv + f * A.out_fs : nullptr;
    const float omega = A.omega, one_m_omega = 1.0f - omega, wa = A.wa, wb = A.wb;
    const bool row_ok = r < h;
    const bool has_below = r + 1 < h;
    const int last = T.n - 1;
    auto span = [&](int pk) {
        const int G_p = pk >> 8;
        return w + (G_p > 1 ? 2 * (G_p - 1) : 1);
    };

    // inputs of the pixel entering at column c of a pass with flags pk, and the
    // pass-start value of the pixel below its left neighbour (fetch of k_sor_regs)
    auto fetch = [&](int c, int pk, Pre<K>& p) {
        const bool zero = (pk & kPkZero) != 0;
        const int o = (r + c) * P;
        if (row_ok && c >= 0 && c < w) {
            if (CO && (pk & kPkCoef)) {
#pragma unroll
                for (int q = 0; q < 5; ++q) p.raw.j[q] = coefr[q * pl + o];
            } else {
#pragma unroll
                for (int q = 0; q < 6 * K; ++q) p.raw.j[q] = Jr[q * pl + o];
#pragma unroll
                for (int k = 0; k < K; ++k) p.raw.w[k] = Wr[k * pl + o];
                p.raw.lu = lapr[o];
                p.raw.lv = lapr[pl + o];
            }
            p.raw.du = zero ? 0.0f : dur[o];
            p.raw.dv = zero ? 0.0f : dvr[o];
        }
        if (has_below && c >= 1 && c <= w) {
            p.nu = zero ? 0.0f : dur[o + 1];
            p.nv = zero ? 0.0f : dvr[o + 1];
        }
    };
    auto fold_into = [&](int c, int pk, const Pre<K>& p, int slot) {
        if (row_ok && c >= 0 && c < w) {
            const Coef cf = fold_pk<K, CO>(A, pk, p.raw);
            if (CO && (pk & kPkStore)) {
                const int o = (r + c) * P;
                coefr[o] = cf.A12;
                coefr[pl + o] = cf.BU;
                coefr[2 * pl + o] = cf.BV;
                coefr[3 * pl + o] = cf.iDu;
                coefr[4 * pl + o] = cf.iDv;
            }
            C4[slot * NT + t] = make_float4(cf.A12, cf.BU, cf.BV, cf.iDu);
            C1[slot * NT + t] = cf.iDv;
        }
    };
    auto xs = [&](int par, int wp, int dir, int gi) -> float2& { return X[((par * NW + wp) * 2 + dir) * G + gi]; };
    auto step_barrier = [&]() {
        if constexpr (CL)
            cooperative_groups::this_cluster().sync();
        else
            __syncthreads();
    };
    if constexpr (CL) step_barrier();  // every CTA of the cluster is running before any remote write

    // the row's current pass (of the update at tau = s - r): index, local start and
    // end, its flags and those of the next pass; the fold (tau + 1) and the prefetch
    // (tau + 2) fall in the current or the next pass (every span is at least w + 1 >= 4)
    int cp = 0, cstart = 0;
    int pk_cur = T.pk[0];
    int pk_nxt = last > 0 ? T.pk[1] : 0;
    int cend = span(pk_cur);
    Pre<K> pre[2];
    fetch(-r, pk_cur, pre[0]);
    fetch(1 - r, pk_cur, pre[1]);
    fold_into(-r, pk_cur, pre[0], 0);
    float2 V0[G], V1[G], V2[G];
#pragma unroll
    for (int gi = 0; gi < G; ++gi) V0[gi] = V1[gi] = V2[gi] = make_float2(0.0f, 0.0f);

    int total = 0;
    for (int p = 0; p < T.n; ++p) total += span(T.pk[p]);
    const int nsteps = total + h - 1;
    int slot0 = 0;  // s % S
    for (int s0 = 0; s0 < nsteps; s0 += 2) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int s = s0 + q;
            if (s < nsteps) {
                Pre<K>& cur = pre[q];       // the pixel entering at step s
                Pre<K>& nxt = pre[q ^ 1];   // the pixel entering at step s + 1
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
                const bool final_rm = !more && odu != nullptr;
                const int c0 = tau - cstart;
                const float2 ps0 = make_float2(cur.raw.du, cur.raw.dv);
                const float2 ps1 = make_float2(nxt.raw.du, nxt.raw.dv);
                const float2 dn1 = make_float2(nxt.nu, nxt.nv);
                fetch(e_nx ? tau + 2 - cend : c0 + 2, e_nx ? pk_nxt : pk_cur, cur);
                const int pin = (s + 1) & 1;  // parity written at step s - 1
#pragma unroll
                for (int gj = 0; gj < G; ++gj) {
                    const int gi = G - 1 - gj;  // the independent updates first, the newest column last
                    float2 up, dn;
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
                        const float2 own = gi == 0 ? ps0 : V2[gi - 1];
                        const float2 lf = c > 0 ? V1[gi] : own;
                        const float2 rt = c < w - 1 ? (gi == 0 ? ps1 : V1[gi - 1]) : own;
                        const float2 u_ = r > 0 ? up : own;
                        const float2 d_ = r < h - 1 ? dn : own;
                        int sl = slot0 - 2 * gi;
                        if (sl < 0) sl += S;
                        V0[gi] = sor_point(own, u_, d_, lf, rt, C4[sl * NT + t], C1[sl * NT + t], wa, wb, omega,
                                           one_m_omega);
                        if (gi == Gp - 1) {
                            if (final_rm) {
                                odu[r * w + c] = V0[gi].x;
                                odv[r * w + c] = V0[gi].y;
                            } else {
                                dur[(r + c) * P] = V0[gi].x;
                                dvr[(r + c) * P] = V0[gi].y;
                            }
                        }
                    }
                }
                fold_into(f_nx ? tau + 1 - cend : c0 + 1, f_nx ? pk_nxt : pk_cur, nxt, slot1);
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
                    // strip edges: the last row feeds the next strip's "up", the first row the
                    // previous strip's "down", in the neighbouring CTA's shared memory
                    if (t == NT - 1 && strip < nc - 1) {
                        float2* dst = cooperative_groups::this_cluster().map_shared_rank(XE, strip + 1);
#pragma unroll
                        for (int gi = 0; gi < G; ++gi) dst[(pout * 2 + 0) * G + gi] = V0[gi];
                    }
                    if (t == 0 && strip > 0) {
                        float2* dst = cooperative_groups::this_cluster().map_shared_rank(XE, strip - 1);
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

constexpr int kSmemLimit = 232448;  // 227 KB of dynamic shared memory per CTA

template <int K, int PF, int MAXT>
cudaError_t run_fused_t(const SorArgs& A, int n_frames, int threads, cudaStream_t st)
{
    {
        const cudaError_t e = ensure_max_dyn_smem((const void*)k_sor_fused<K, PF, MAXT>, kSmemLimit);
        if (e != cudaSuccess) return e;
    }
    const size_t smem = (size_t)(2 * A.G + 3) * 7 * A.g.P * sizeof(float);
    k_sor_fused<K, PF, MAXT><<<n_frames, threads, smem, st>>>(A);
    return cudaGetLastError();
}

// threads per CTA: at least the rows of the longest diagonal (P), at most
// 1024.  Up to 512 threads: the variant with registers for 512 threads and
// the deeper prefetch; above: the 1024-thread variant.
template <int K, int PF>
cudaError_t run_fused(const SorArgs& A, int n_frames, int threads, cudaStream_t st)
{
    if (threads <= kMaxLane) return run_fused_t<K, PF, kMaxLane>(A, n_frames, threads, st);
    return run_fused_t<K, 1, 2 * kMaxLane>(A, n_frames, threads, st);
}

}  // namespace

bool sor_fused_supports(int K) { return K >= 1 && K <= 4; }

int sor_fused_gmax(int P)
{
    if (P > 2 * kMaxLane) return 0;
    for (int G = kGMax; G >= 1; --G)
        if ((size_t)(2 * G + 3) * 7 * P * sizeof(float) <= (size_t)kSmemLimit) return G;
    return 0;
}

size_t sor_regs_smem(int G, int threads)
{
    return (size_t)(2 * G - 1) * 5 * threads * sizeof(float) +
           (size_t)(2 * (threads / 32) * 2 * G + 2 * 2 * G) * sizeof(float2);
}

// Row strips of a level: one CTA when it has at most 512 rows, else a cluster of
// nc <= 8 CTAs of NT rows each (K <= 2: the registers of the larger K leave no room).
static void regs_split(int K, const DiagGeom& g, int* nc, int* nt)
{
    if (g.P <= kMaxLane) {
        *nc = 1;
        *nt = g.P;
        return;
    }
    const int n = (g.P + kMaxLane - 1) / kMaxLane;
    *nc = (K <= 2 && n <= 8) ? n : 0;
    *nt = ((g.P + n - 1) / n + 31) / 32 * 32;
}

bool sor_regs_supports(int K, const DiagGeom& g)
{
    int nc, nt;
    regs_split(K, g, &nc, &nt);
    return K >= 1 && K <= 4 && (g.P & 31) == 0 && nc >= 1;
}

namespace {

template <int K, int G>
cudaError_t run_regs_t(const SorArgs& A, int n_frames, int nt, cudaStream_t st)
{
    if (A.nc == 1) {
        {
            const cudaError_t e = ensure_max_dyn_smem((const void*)k_sor_regs<K, G, false>, kSmemLimit);
            if (e != cudaSuccess) return e;
        }
        k_sor_regs<K, G, false><<<n_frames, nt, sor_regs_smem(G, nt), st>>>(A);
        return cudaGetLastError();
    }
    if constexpr (K <= 2) {
        {
            const cudaError_t e = ensure_max_dyn_smem((const void*)k_sor_regs<K, G, true>, kSmemLimit);
            if (e != cudaSuccess) return e;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(n_frames * A.nc));
        cfg.blockDim = dim3((unsigned)nt);
        cfg.dynamicSmemBytes = sor_regs_smem(G, nt);
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)A.nc;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_sor_regs<K, G, true>, A);
    } else {
        return cudaErrorInvalidValue;
    }
}

template <int K>
cudaError_t run_regs(const SorArgs& A, int n_frames, int nt, cudaStream_t st)
{
    switch (A.G) {
        case 1: return run_regs_t<K, 1>(A, n_frames, nt, st);
        case 2: return run_regs_t<K, 2>(A, n_frames, nt, st);
        case 3: return run_regs_t<K, 3>(A, n_frames, nt, st);
        case 4: return run_regs_t<K, 4>(A, n_frames, nt, st);
        default: return run_regs_t<K, 5>(A, n_frames, nt, st);
    }
}

SorArgs make_args(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap, long long lap_fs,
                  float* coef, long long coef_fs, float* du, float* dv, long long st_fs, int K, DiagGeom g, int G,
                  int mode, int store_coef, const float* a_data, float wx, float wy, float omega, float* out_du,
                  float* out_dv, long long out_fs)
{
    SorArgs A;
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
    A.g = g;
    A.G = G;
    A.mode = mode;
    A.store_coef = store_coef;
    A.wa = wy;  // the lane index runs along rows: row neighbours carry the y weight
    A.wb = wx;
    A.wsum = ((wx + wx) + wy) + wy;
    A.omega = omega;
    for (int k = 0; k < kMaxK; ++k) A.a_data[k] = k < K ? a_data[k] : 0.0f;
    A.nc = 1;
    return A;
}

}  // namespace

cudaError_t launch_sor_regs(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap,
                            long long lap_fs, float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                            int n_frames, int K, DiagGeom g, int G, int mode, int store_coef, const float* a_data,
                            float wx, float wy, float omega, cudaStream_t st, float* out_du, float* out_dv,
                            long long out_fs)
{
    int nc = 0, nt = 0;
    regs_split(K, g, &nc, &nt);
    if (G < 1 || G > kGMax || !sor_regs_supports(K, g) || sor_regs_smem(G, nt) > (size_t)kSmemLimit ||
        (long long)n_frames * nc > 0x7fffffffLL)
        return cudaErrorInvalidValue;
    SorArgs A = make_args(J, J_fs, W, W_fs, lap, lap_fs, coef, coef_fs, du, dv, st_fs, K, g, G, mode, store_coef,
                          a_data, wx, wy, omega, out_du, out_dv, out_fs);
    A.nc = nc;
    switch (K) {
        case 1: return run_regs<1>(A, n_frames, nt, st);
        case 2: return run_regs<2>(A, n_frames, nt, st);
        case 3: return run_regs<3>(A, n_frames, nt, st);
        default: return run_regs<4>(A, n_frames, nt, st);
    }
}

namespace {

template <int K, int G, bool CO>
cudaError_t run_chain_t(const SorArgs& A, const ChainTable& T, int n_frames, int nt, cudaStream_t st)
{
    if (A.nc == 1) {
        {
            const cudaError_t e = ensure_max_dyn_smem((const void*)k_sor_chain<K, G, CO, false>, kSmemLimit);
            if (e != cudaSuccess) return e;
        }
        k_sor_chain<K, G, CO, false><<<n_frames, nt, sor_regs_smem(G, nt), st>>>(A, T);
        return cudaGetLastError();
    }
    if constexpr (K <= 2) {
        {
            const cudaError_t e = ensure_max_dyn_smem((const void*)k_sor_chain<K, G, CO, true>, kSmemLimit);
            if (e != cudaSuccess) return e;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(n_frames * A.nc));
        cfg.blockDim = dim3((unsigned)nt);
        cfg.dynamicSmemBytes = sor_regs_smem(G, nt);
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = (unsigned)A.nc;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_sor_chain<K, G, CO, true>, A, T);
    } else {
        return cudaErrorInvalidValue;
    }
}

template <int K, bool CO>
cudaError_t run_chain_c(const SorArgs& A, const ChainTable& T, int gmax, int n_frames, int nt, cudaStream_t st)
{
    switch (gmax) {
        case 1: return run_chain_t<K, 1, CO>(A, T, n_frames, nt, st);
        case 2: return run_chain_t<K, 2, CO>(A, T, n_frames, nt, st);
        case 3: return run_chain_t<K, 3, CO>(A, T, n_frames, nt, st);
        case 4: return run_chain_t<K, 4, CO>(A, T, n_frames, nt, st);
        default: return run_chain_t<K, 5, CO>(A, T, n_frames, nt, st);
    }
}

// CO: some pass reads back or stores folded coefficients (windows between psi
// ticks longer than the pass length)
template <int K>
cudaError_t run_chain(const SorArgs& A, const ChainTable& T, bool co, int gmax, int n_frames, int nt,
                      cudaStream_t st)
{
    return co ? run_chain_c<K, true>(A, T, gmax, n_frames, nt, st) : run_chain_c<K, false>(A, T, gmax, n_frames, nt, st);
}

}  // namespace

bool sor_chain_supports(int K, const DiagGeom& g, int n_passes)
{
    // 32-bit offsets: the largest plane index read is (6K + 2) planes of D * P
    const long long plane = (long long)g.D * g.P;
    return sor_regs_supports(K, g) && g.w >= 3 && n_passes >= 1 && n_passes <= kMaxChain &&
           plane * (6 * K + 2) < 0x7fffffffLL && (long long)g.h * g.w < 0x7fffffffLL;
}

cudaError_t launch_sor_chain(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap,
                             long long lap_fs, float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                             int n_frames, int K, DiagGeom g, const ChainPass* passes, int n_passes,
                             const float* a_data, float wx, float wy, float omega, cudaStream_t st, float* out_du,
                             float* out_dv, long long out_fs)
{
    int nc = 0, nt = 0;
    regs_split(K, g, &nc, &nt);
    if (!sor_chain_supports(K, g, n_passes) || n_frames < 1 || (long long)n_frames * nc > 0x7fffffffLL)
        return cudaErrorInvalidValue;
    ChainTable T;
    T.n = n_passes;
    int gmax = 1;
    bool co = false;
    for (int p = 0; p < n_passes; ++p) {
        const ChainPass& q = passes[p];
        if (q.G < 1 || q.G > kGMax || q.mode < -1 || q.mode > 3) return cudaErrorInvalidValue;
        const bool coef = q.mode < 0, store = q.mode >= 0 && q.store_coef;
        T.pk[p] = (q.G << 8) | (store ? kPkStore : 0) | (coef ? kPkCoef : 0) |
                  (!coef && (q.mode & 2) ? kPkTick : 0) | (!coef && (q.mode & 1) ? kPkZero : 0);
        co = co || coef || store;
        gmax = q.G > gmax ? q.G : gmax;
    }
    for (int p = n_passes; p < kMaxChain; ++p) T.pk[p] = 1 << 8;
    if (sor_regs_smem(gmax, nt) > (size_t)kSmemLimit) return cudaErrorInvalidValue;
    SorArgs A = make_args(J, J_fs, W, W_fs, lap, lap_fs, coef, coef_fs, du, dv, st_fs, K, g, gmax, 0, 0, a_data, wx,
                          wy, omega, out_du, out_dv, out_fs);
    A.nc = nc;
    switch (K) {
        case 1: return run_chain<1>(A, T, co, gmax, n_frames, nt, st);
        case 2: return run_chain<2>(A, T, co, gmax, n_frames, nt, st);
        case 3: return run_chain<3>(A, T, co, gmax, n_frames, nt, st);
        default: return run_chain<4>(A, T, co, gmax, n_frames, nt, st);
    }
}

cudaError_t launch_sor_fused(const float* J, long long J_fs, const float* W, long long W_fs, const float* lap,
                             long long lap_fs, float* coef, long long coef_fs, float* du, float* dv, long long st_fs,
                             int n_frames, int K, DiagGeom g, int G, int mode, int store_coef, const float* a_data,
                             float wx, float wy, float omega, cudaStream_t st, float* out_du, float* out_dv,
                             long long out_fs, int threads)
{
    if (G < 1 || G > sor_fused_gmax(g.P) || (g.P & 31) || !sor_fused_supports(K)) return cudaErrorInvalidValue;
    if (threads <= 0) threads = g.P;
    if (threads < g.P || threads > 2 * kMaxLane || (threads & 31)) return cudaErrorInvalidValue;
    SorArgs A;
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
    A.g = g;
    A.G = G;
    A.mode = mode;
    A.store_coef = store_coef;
    A.wa = wy;  // the lane index runs along rows: row neighbours carry the y weight
    A.wb = wx;
    A.wsum = ((wx + wx) + wy) + wy;
    A.omega = omega;
    for (int k = 0; k < kMaxK; ++k) A.a_data[k] = k < K ? a_data[k] : 0.0f;
    switch (K) {
        case 1: return run_fused<1, 2>(A, n_frames, threads, st);
        case 2: return run_fused<2, 2>(A, n_frames, threads, st);
        case 3: return run_fused<3, 1>(A, n_frames, threads, st);
        default: return run_fused<4, 1>(A, n_frames, threads, st);
    }
}

}  // namespace frg
