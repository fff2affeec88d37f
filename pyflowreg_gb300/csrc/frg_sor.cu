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

// fold (or pass the stored coefficients through) and store into ring row a
template <int K>
__device__ __forceinline__ void put_raw(const SorArgs& A, const Raw<K>& r, float2* DV, float4* C4, float* C1, int a,
                                        float* coef, long long o, long long plane)
{
    float A12, BU, BV, iDu, iDv;
    if (A.mode < 0) {
        A12 = r.j[0];
        BU = r.j[1];
        BV = r.j[2];
        iDu = r.j[3];
        iDv = r.j[4];
    } else {
        const bool tick = (A.mode & 2) != 0;
        float A11 = 0.f, A22 = 0.f, a12 = 0.f, C13 = 0.f, C23 = 0.f;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float j11 = r.j[0 * K + k], j22 = r.j[1 * K + k], j33 = r.j[2 * K + k];
            const float j12 = r.j[3 * K + k], j13 = r.j[4 * K + k], j23 = r.j[5 * K + k];
            float psi = 1.0f;
            if (tick) {
                const float a = r.du, b = r.dv;
                float E = j11 * a * a + j22 * b * b + j23 * b + 2.0f * j12 * a * b + 2.0f * j13 * a + j23 * b + j33;
                E = fmaxf(E, 0.0f);
                // (E + eps)^(a_k - 1) as exp2((a_k - 1) log2(E + eps)) on the special-function
                // unit: relative error ~1e-6, the fp32 path's rounding level
                psi = A.a_data[k] * exp2f((A.a_data[k] - 1.0f) * __log2f(E + 1e-5f));
            }
            const float wp = r.w[k] * psi;
            A11 = fmaf(wp, j11, A11);
            A22 = fmaf(wp, j22, A22);
            a12 = fmaf(wp, j12, a12);
            C13 = fmaf(wp, j13, C13);
            C23 = fmaf(wp, j23, C23);
        }
        const float den_u = A.wsum + A11, den_v = A.wsum + A22;
        A12 = a12;
        BU = r.lu - C13;
        BV = r.lv - C23;
        iDu = den_u != 0.0f ? __frcp_rn(den_u) : 0.0f;
        iDv = den_v != 0.0f ? __frcp_rn(den_v) : 0.0f;
        if (A.store_coef) {
            coef[o] = A12;
            coef[plane + o] = BU;
            coef[2 * plane + o] = BV;
            coef[3 * plane + o] = iDu;
            coef[4 * plane + o] = iDv;
        }
    }
    DV[a] = make_float2(r.du, r.dv);
    C4[a] = make_float4(A12, BU, BV, iDu);
    C1[a] = iDv;
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
                    const float nu = wa * (am.x + ap.x) + wb * (bm.x + bp.x) + c4.y - c4.x * c.y;
                    const float dun = one_m_omega * c.x + omega * (nu * c4.w);
                    const float nv = wa * (am.y + ap.y) + wb * (bm.y + bp.y) + c4.z - c4.x * dun;
                    const float dvn = one_m_omega * c.y + omega * (nv * iDv);
                    DVc[a] = make_float2(dun, dvn);
                }
                if (++slot_s == R) slot_s = 0;
            }
            __syncthreads();
        }
    }
    for (int e = nsteps - 2 * G > 0 ? nsteps - 2 * G : 0; e < D; ++e) writeback(e, e % R);
}

constexpr int kSmemLimit = 232448;  // 227 KB of dynamic shared memory per CTA

template <int K, int PF, int MAXT>
cudaError_t run_fused_t(const SorArgs& A, int n_frames, int threads, cudaStream_t st)
{
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_sor_fused<K, PF, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmemLimit);
        if (e != cudaSuccess) return e;
        attr = true;
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
