/*
 * flowreg_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A CPU restatement, in plain C, of pyflowreg's variational optical-flow path
 * (get_displacement, single stage, no GNC).  It exists to check the GB300
 * kernels and to serve as the timed CPU baseline; the product never links,
 * loads or calls it.  Every function cites the reference lines it follows
 * (paths relative to pyflowreg's src/pyflowreg/).
 *
 * Arithmetic follows the reference as executed by numpy/Python semantics:
 *   - resize: float32 data and tables, products rounded to float32, float64
 *     accumulator, float32 output (util/resize_util.py:116-141, 232-254);
 *   - warp: the cv2.remap bicubic/bilinear rules on a 1/32-pixel grid, float32
 *     weights, double accumulation on the float64 level image, float32 output
 *     (core/warping.py:160-234);
 *   - motion tensor: float64, except that terms differentiated from the warped
 *     image are computed in float32 exactly where numpy does so (the warped
 *     image is a float32 array at every level below the top);
 *   - level solver: float64, lexicographic column-major SOR exactly as
 *     core/level_solver.py:158-369, or (order = 1) red-black ordering with the
 *     same per-pixel arithmetic, for measuring the ordering gap;
 *   - median: 5x5, scipy.ndimage "mirror" boundary (core/optical_flow.py:607-609).
 *
 * Build: oracle/build_oracle.sh (gcc -O2 -fno-fast-math -ffp-contract=off).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* ------------------------------------------------------------------------ */
/* Fused Gauss-cubic resize passes: util/resize_util.py:116-141              */
/* src/dst are float32 planes, row-major.                                    */
/* ------------------------------------------------------------------------ */
/* acc_f32 = 0: numba typing (the reference as deployed): the accumulator `s`
 * is float64.  acc_f32 = 1: the same source executed as plain Python under
 * numpy 2 promotion rules, where `0.0 + float32` stays float32 (used only to
 * pin against golden vectors produced by running the reference source
 * without numba). */
void orc_resize_plane(const float *src, int ih, int iw, float *dst, int oh, int ow,
                      const int32_t *ix, const float *wx, int px,
                      const int32_t *iy, const float *wy, int py, float *tmp /* ih*ow */,
                      int acc_f32)
{
    /* _resize_h: dst[y, x] = sum_p f32(src[y, idx[x,p]] * wt[x,p]) */
    for (int y = 0; y < ih; ++y) {
        const float *row = src + (size_t)y * iw;
        for (int x = 0; x < ow; ++x) {
            double s = 0.0;
            float sf = 0.0f;
            for (int p = 0; p < px; ++p) {
                float prod = row[ix[x * px + p]] * wx[x * px + p];
                s += (double)prod;
                sf += prod;
            }
            tmp[(size_t)y * ow + x] = acc_f32 ? sf : (float)s;
        }
    }
    /* _resize_v */
    for (int x = 0; x < ow; ++x) {
        for (int y = 0; y < oh; ++y) {
            double s = 0.0;
            float sf = 0.0f;
            for (int p = 0; p < py; ++p) {
                float prod = tmp[(size_t)iy[y * py + p] * ow + x] * wy[y * py + p];
                s += (double)prod;
                sf += prod;
            }
            dst[(size_t)y * ow + x] = acc_f32 ? sf : (float)s;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* cv2.remap weights at 1/32 positions (documented Keys A=-0.75 / bilinear). */
/* ------------------------------------------------------------------------ */
static float keys_inner(float x)
{
    const float A = -0.75f;
    float a = (A + 2.0f) * x;
    a = a - (A + 3.0f);
    float xx = x * x;
    a = a * xx;
    return a + 1.0f;
}

static float keys_outer(float x)
{
    const float A = -0.75f;
    float t = A * x - 5.0f * A;
    t = t * x + 8.0f * A;
    return t * x - 4.0f * A;
}

void orc_cubic_table(float *tab /* 32*4 */)
{
    for (int k = 0; k < 32; ++k) {
        float t = (float)k / 32.0f;
        float w0 = keys_outer(1.0f + t);
        float w1 = keys_inner(t);
        float w2 = keys_inner(1.0f - t);
        float w3 = ((1.0f - w0) - w1) - w2;
        tab[k * 4 + 0] = w0;
        tab[k * 4 + 1] = w1;
        tab[k * 4 + 2] = w2;
        tab[k * 4 + 3] = w3;
    }
}

void orc_linear_table(float *tab /* 32*2 */)
{
    for (int k = 0; k < 32; ++k) {
        float t = (float)k / 32.0f;
        tab[k * 2 + 0] = 1.0f - t;
        tab[k * 2 + 1] = t;
    }
}

/* round half to even of a double holding an exact multiple-of-1/32 product */
static inline long long rint_even(double x) { return (long long)nearbyint(x); }

/*
 * imregister_wrapper for one channel: core/warping.py:160-234.
 * f2, f1: level planes (h x w) in double; u, v: displacement in level pixels
 * (already divided by the grid spacings), double.  Output rounded to float32.
 * cubic != 0: bicubic, else bilinear.
 */
void orc_warp_plane(const double *f2, const double *f1, const double *u, const double *v,
                    int h, int w, int cubic, float *out)
{
    float ctab[32 * 4], ltab[32 * 2];
    orc_cubic_table(ctab);
    orc_linear_table(ltab);
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t o = (size_t)y * w + x;
            float mx = (float)((double)x + u[o]);
            float my = (float)((double)y + v[o]);
            int oob = (mx < 0.0f) || (mx >= (float)w) || (my < 0.0f) || (my >= (float)h);
            if (oob) {
                out[o] = (float)f1[o];
                continue;
            }
            float cx = mx < 0.0f ? 0.0f : (mx > (float)(w - 1) ? (float)(w - 1) : mx);
            float cy = my < 0.0f ? 0.0f : (my > (float)(h - 1) ? (float)(h - 1) : my);
            long long X = rint_even((double)cx * 32.0);
            long long Y = rint_even((double)cy * 32.0);
            int ix = (int)(X >> 5), fx = (int)(X & 31);
            int iy = (int)(Y >> 5), fy = (int)(Y & 31);
            double acc = 0.0;
            if (cubic) {
                for (int i = 0; i < 4; ++i) {
                    int yy = clampi(iy - 1 + i, 0, h - 1);
                    for (int j = 0; j < 4; ++j) {
                        int xx = clampi(ix - 1 + j, 0, w - 1);
                        float w2d = ctab[fy * 4 + i] * ctab[fx * 4 + j];
                        acc += f2[(size_t)yy * w + xx] * (double)w2d;
                    }
                }
            } else {
                for (int i = 0; i < 2; ++i) {
                    int yy = clampi(iy + i, 0, h - 1);
                    for (int j = 0; j < 2; ++j) {
                        int xx = clampi(ix + j, 0, w - 1);
                        float w2d = ltab[fy * 2 + i] * ltab[fx * 2 + j];
                        acc += f2[(size_t)yy * w + xx] * (double)w2d;
                    }
                }
            }
            out[o] = (float)acc;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Motion tensors: core/optical_flow.py:73-160 (gc), 163-228 (gray).         */
/* f1: double plane; f2: double plane whose values are float32 when          */
/* f2_is_f32 (then numpy differentiates it in float32).                      */
/* Outputs: six (h+2) x (w+2) double planes, zero ring.                      */
/* ------------------------------------------------------------------------ */

/* numpy.gradient along x of an edge-padded (h+2)x(w+2) array, one entry. */
static inline double grad_x_d(const double *p, int W2, int y, int x, double hx)
{
    if (x == 0) return (p[y * W2 + 1] - p[y * W2 + 0]) / hx;
    if (x == W2 - 1) return (p[y * W2 + x] - p[y * W2 + x - 1]) / hx;
    return (p[y * W2 + x + 1] - p[y * W2 + x - 1]) / (2.0 * hx);
}

static inline double grad_y_d(const double *p, int H2, int W2, int y, int x, double hy)
{
    if (y == 0) return (p[W2 + x] - p[x]) / hy;
    if (y == H2 - 1) return (p[y * W2 + x] - p[(y - 1) * W2 + x]) / hy;
    return (p[(y + 1) * W2 + x] - p[(y - 1) * W2 + x]) / (2.0 * hy);
}

static inline float grad_x_f(const float *p, int W2, int y, int x, float hx_f, float h2x_f)
{
    if (x == 0) return (p[y * W2 + 1] - p[y * W2 + 0]) / hx_f;
    if (x == W2 - 1) return (p[y * W2 + x] - p[y * W2 + x - 1]) / hx_f;
    return (p[y * W2 + x + 1] - p[y * W2 + x - 1]) / h2x_f;
}

static inline float grad_y_f(const float *p, int H2, int W2, int y, int x, float hy_f, float h2y_f)
{
    if (y == 0) return (p[W2 + x] - p[x]) / hy_f;
    if (y == H2 - 1) return (p[y * W2 + x] - p[(y - 1) * W2 + x]) / hy_f;
    return (p[(y + 1) * W2 + x] - p[(y - 1) * W2 + x]) / h2y_f;
}

/* symmetric pad by one of an h x w plane == edge pad by one */
static void pad1_d(const double *f, int h, int w, double *p)
{
    int W2 = w + 2;
    for (int y = 0; y < h + 2; ++y) {
        int sy = clampi(y - 1, 0, h - 1);
        for (int x = 0; x < W2; ++x) p[y * W2 + x] = f[(size_t)sy * w + clampi(x - 1, 0, w - 1)];
    }
}

/* re-pad: keep interior of a (h+2)x(w+2) array, replace the ring by edge copies */
static void repad_d(double *p, int h, int w)
{
    int W2 = w + 2, H2 = h + 2;
    for (int x = 1; x <= w; ++x) {
        p[x] = p[W2 + x];
        p[(H2 - 1) * W2 + x] = p[(H2 - 2) * W2 + x];
    }
    for (int y = 0; y < H2; ++y) {
        p[y * W2] = p[y * W2 + 1];
        p[y * W2 + W2 - 1] = p[y * W2 + W2 - 2];
    }
}

/* Census tensor (core/optical_flow.py:231-345) with numpy's dtypes: f1 is float64; f2 is
 * float32 when f2_is_f32, and then the directional difference, the smoothed Heaviside and its
 * gradient are float32 (Python-float constants cast to float32); the J sums are float64. */
static int census_tensor(const double *f1, const double *f2, int h, int w, double hy, double hx,
                         int f2_is_f32, double *J11, double *J22, double *J33, double *J12,
                         double *J13, double *J23)
{
    const double eps = 0.1 / 255.0, eps2 = eps * eps;
    const int H2 = h + 2, W2 = w + 2;
    const size_t N = (size_t)H2 * W2;
    double *f1p = malloc(N * sizeof(double)), *f2p = malloc(N * sizeof(double));
    double *s1p = malloc(N * sizeof(double)), *s2p = malloc(N * sizeof(double));
    float *s2pf = malloc(N * sizeof(float));
    if (!f1p || !f2p || !s1p || !s2p || !s2pf) {
        free(f1p); free(f2p); free(s1p); free(s2p); free(s2pf);
        return ORC_ENOMEM;
    }
    pad1_d(f1, h, w, f1p);
    pad1_d(f2, h, w, f2p);
    memset(J11, 0, N * sizeof(double)); memset(J22, 0, N * sizeof(double));
    memset(J33, 0, N * sizeof(double)); memset(J12, 0, N * sizeof(double));
    memset(J13, 0, N * sizeof(double)); memset(J23, 0, N * sizeof(double));
    const float eps2f = (float)eps2, h2x_f = (float)(2.0 * hx), h2y_f = (float)(2.0 * hy);
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            if (dy == 0 && dx == 0) continue;
            const double dist = sqrt((hy * dy) * (hy * dy) + (hx * dx) * (hx * dx));
            const float dist_f = (float)dist;
            /* core values s(y, x), y < h, x < w, written edge-padded into s1p / s2p */
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x) {
                    const size_t c = (size_t)(y + 1) * W2 + (x + 1);
                    const size_t nb = (size_t)(y + 1 + dy) * W2 + (x + 1 + dx);
                    const double r1 = (f1p[nb] - f1p[c]) / dist;
                    const double s1 = 0.5 * (1.0 + r1 / sqrt(r1 * r1 + eps2));
                    double s2;
                    if (f2_is_f32) {
                        const float d = (float)f2p[nb] - (float)f2p[c];
                        const float r2 = d / dist_f;
                        const float q = sqrtf(r2 * r2 + eps2f);
                        s2 = (double)(0.5f * (1.0f + r2 / q));
                    } else {
                        const double r2 = (f2p[nb] - f2p[c]) / dist;
                        s2 = 0.5 * (1.0 + r2 / sqrt(r2 * r2 + eps2));
                    }
                    s1p[c] = s1;
                    s2p[c] = s2;
                }
            for (int y = 0; y < H2; ++y)
                for (int x = 0; x < W2; ++x) {
                    const size_t o = (size_t)y * W2 + x;
                    const size_t src = (size_t)clampi(y, 1, h) * W2 + clampi(x, 1, w);
                    s1p[o] = s1p[src];
                    s2p[o] = s2p[src];
                }
            for (size_t i = 0; i < N; ++i) s2pf[i] = (float)s2p[i];
            for (int y = 1; y <= h; ++y)
                for (int x = 1; x <= w; ++x) {
                    const size_t o = (size_t)y * W2 + x;
                    const double sx1 = (s1p[o + 1] - s1p[o - 1]) / (2.0 * hx);
                    const double sy1 = (s1p[o + W2] - s1p[o - W2]) / (2.0 * hy);
                    double sx2, sy2;
                    if (f2_is_f32) {
                        sx2 = (double)((s2pf[o + 1] - s2pf[o - 1]) / h2x_f);
                        sy2 = (double)((s2pf[o + W2] - s2pf[o - W2]) / h2y_f);
                    } else {
                        sx2 = (s2p[o + 1] - s2p[o - 1]) / (2.0 * hx);
                        sy2 = (s2p[o + W2] - s2p[o - W2]) / (2.0 * hy);
                    }
                    const double sx = 0.5 * (sx1 + sx2), sy = 0.5 * (sy1 + sy2);
                    const double st = s2p[o] - s1p[o];
                    J11[o] += sx * sx; J22[o] += sy * sy; J33[o] += st * st;
                    J12[o] += sx * sy; J13[o] += sx * st; J23[o] += sy * st;
                }
        }
    const double scale = 2.0 / 8.0;
    for (int y = 1; y <= h; ++y)
        for (int x = 1; x <= w; ++x) {
            const size_t o = (size_t)y * W2 + x;
            J11[o] *= scale; J22[o] *= scale; J33[o] *= scale;
            J12[o] *= scale; J13[o] *= scale; J23[o] *= scale;
        }
    free(f1p); free(f2p); free(s1p); free(s2p); free(s2pf);
    return ORC_OK;
}

int orc_motion_tensor(const double *f1, const double *f2, int h, int w, double hy, double hx,
                      int f2_is_f32, int gray, double *J11, double *J22, double *J33,
                      double *J12, double *J13, double *J23)
{
    if (gray == 2)
        return census_tensor(f1, f2, h, w, hy, hx, f2_is_f32, J11, J22, J33, J12, J13, J23);
    int H2 = h + 2, W2 = w + 2;
    size_t N = (size_t)H2 * W2;
    double *f1p = malloc(N * sizeof(double));
    double *f2p = malloc(N * sizeof(double));
    float *f2pf = malloc(N * sizeof(float));
    double *gx1 = malloc(N * sizeof(double)), *gx2 = malloc(N * sizeof(double));
    double *gy1 = malloc(N * sizeof(double)), *gy2 = malloc(N * sizeof(double));
    double *fx = malloc(N * sizeof(double)), *fy = malloc(N * sizeof(double));
    double *ft = malloc(N * sizeof(double));
    if (!f1p || !f2p || !f2pf || !gx1 || !gx2 || !gy1 || !gy2 || !fx || !fy || !ft) {
        free(f1p); free(f2p); free(f2pf); free(gx1); free(gx2); free(gy1); free(gy2);
        free(fx); free(fy); free(ft);
        return ORC_ENOMEM;
    }
    pad1_d(f1, h, w, f1p);
    pad1_d(f2, h, w, f2p);
    for (size_t i = 0; i < N; ++i) f2pf[i] = (float)f2p[i];
    /* numpy casts the Python-float spacing to float32 for float32 operands */
    float hx_f = (float)hx, hy_f = (float)hy, h2x_f = (float)(2.0 * hx), h2y_f = (float)(2.0 * hy);
    float hxx_f = (float)(hx * hx), hyy_f = (float)(hy * hy);

    for (int y = 0; y < H2; ++y)
        for (int x = 0; x < W2; ++x) {
            size_t o = (size_t)y * W2 + x;
            gx1[o] = grad_x_d(f1p, W2, y, x, hx);
            gy1[o] = grad_y_d(f1p, H2, W2, y, x, hy);
            if (f2_is_f32) {
                gx2[o] = (double)grad_x_f(f2pf, W2, y, x, hx_f, h2x_f);
                gy2[o] = (double)grad_y_f(f2pf, H2, W2, y, x, hy_f, h2y_f);
            } else {
                gx2[o] = grad_x_d(f2p, W2, y, x, hx);
                gy2[o] = grad_y_d(f2p, H2, W2, y, x, hy);
            }
            fx[o] = 0.5 * (gx1[o] + gx2[o]);
            fy[o] = 0.5 * (gy1[o] + gy2[o]);
            ft[o] = f2p[o] - f1p[o];
        }
    repad_d(fx, h, w);
    repad_d(fy, h, w);
    repad_d(ft, h, w);

    memset(J11, 0, N * sizeof(double)); memset(J22, 0, N * sizeof(double));
    memset(J33, 0, N * sizeof(double)); memset(J12, 0, N * sizeof(double));
    memset(J13, 0, N * sizeof(double)); memset(J23, 0, N * sizeof(double));

    for (int y = 1; y < H2 - 1; ++y)
        for (int x = 1; x < W2 - 1; ++x) {
            size_t o = (size_t)y * W2 + x;
            if (gray) {
                /* core/optical_flow.py:201-228 */
                double a = fx[o], b = fy[o], c = ft[o];
                J11[o] = a * a; J22[o] = b * b; J33[o] = c * c;
                J12[o] = a * b; J13[o] = a * c; J23[o] = b * c;
                continue;
            }
            /* core/optical_flow.py:119-160 */
            double fxy = grad_y_d(fx, H2, W2, y, x, hy);
            double fxt = grad_x_d(ft, W2, y, x, hx);
            double fyt = grad_y_d(ft, H2, W2, y, x, hy);
            /* gradient2 (lines 134-139): ((f[x-1] - 2 f[x]) + f[x+1]) / h^2 */
            double fxx1 = ((f1p[o - 1] - 2.0 * f1p[o]) + f1p[o + 1]) / (hx * hx);
            double fyy1 = ((f1p[o - W2] - 2.0 * f1p[o]) + f1p[o + W2]) / (hy * hy);
            double fxx2, fyy2;
            if (f2_is_f32) {
                fxx2 = (double)(((f2pf[o - 1] - 2.0f * f2pf[o]) + f2pf[o + 1]) / hxx_f);
                fyy2 = (double)(((f2pf[o - W2] - 2.0f * f2pf[o]) + f2pf[o + W2]) / hyy_f);
            } else {
                fxx2 = ((f2p[o - 1] - 2.0 * f2p[o]) + f2p[o + 1]) / (hx * hx);
                fyy2 = ((f2p[o - W2] - 2.0 * f2p[o]) + f2p[o + W2]) / (hy * hy);
            }
            double fxx = 0.5 * (fxx1 + fxx2);
            double fyy = 0.5 * (fyy1 + fyy2);
            double sx = sqrt(fxx * fxx + fxy * fxy);
            double sy = sqrt(fxy * fxy + fyy * fyy);
            double reg_x = 1.0 / ((sx * sx) + 1e-6);
            double reg_y = 1.0 / ((sy * sy) + 1e-6);
            J11[o] = reg_x * (fxx * fxx) + reg_y * (fxy * fxy);
            J22[o] = reg_x * (fxy * fxy) + reg_y * (fyy * fyy);
            J33[o] = reg_x * (fxt * fxt) + reg_y * (fyt * fyt);
            J12[o] = reg_x * fxx * fxy + reg_y * fxy * fyy;
            J13[o] = reg_x * fxx * fxt + reg_y * fxy * fyt;
            J23[o] = reg_x * fxy * fxt + reg_y * fyy * fyt;
        }
    free(f1p); free(f2p); free(f2pf); free(gx1); free(gx2); free(gy1); free(gy2);
    free(fx); free(fy); free(ft);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Level solver: core/level_solver.py:45-369.                                */
/* J* and weight: (m, n, K) C-contiguous; u, v, du, dv: (m, n).              */
/* order 0: lexicographic (columns outer, rows inner, in place) as numba.    */
/* order 1: red-black ((i + j) even first), same per-pixel arithmetic.       */
/* ------------------------------------------------------------------------ */
static void set_boundary_2d(double *f, int m, int n)
{
    for (int i = 0; i < n; ++i) {
        f[i] = f[n + i];
        f[(size_t)(m - 1) * n + i] = f[(size_t)(m - 2) * n + i];
    }
    for (int j = 0; j < m; ++j) {
        f[(size_t)j * n] = f[(size_t)j * n + 1];
        f[(size_t)j * n + n - 1] = f[(size_t)j * n + n - 2];
    }
}

/* core/level_solver.py:69-155 */
static void nonlinearity_smoothness_2d(double *psi_s, const double *u, const double *du,
                                       const double *v, const double *dv, int m, int n,
                                       double a, double hx, double hy, double *scratch)
{
    const double eps = 0.00001;
    double *uf = scratch, *vf = scratch + (size_t)m * n;
    for (size_t i = 0; i < (size_t)m * n; ++i) {
        uf[i] = u[i] + du[i];
        vf[i] = v[i] + dv[i];
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < m; ++j) {
            double ux = 0, vx = 0, uy = 0, vy = 0;
            size_t o = (size_t)j * n + i;
            if (n > 1) {
                if (i == 0) { ux = (uf[o + 1] - uf[o]) / hx; vx = (vf[o + 1] - vf[o]) / hx; }
                else if (i == n - 1) { ux = (uf[o] - uf[o - 1]) / hx; vx = (vf[o] - vf[o - 1]) / hx; }
                else { ux = (uf[o + 1] - uf[o - 1]) / (2.0 * hx); vx = (vf[o + 1] - vf[o - 1]) / (2.0 * hx); }
            }
            if (m > 1) {
                if (j == 0) { uy = (uf[o + n] - uf[o]) / hy; vy = (vf[o + n] - vf[o]) / hy; }
                else if (j == m - 1) { uy = (uf[o] - uf[o - n]) / hy; vy = (vf[o] - vf[o - n]) / hy; }
                else { uy = (uf[o + n] - uf[o - n]) / (2.0 * hy); vy = (vf[o + n] - vf[o - n]) / (2.0 * hy); }
            }
            double tmp = ux * ux + uy * uy + vx * vx + vy * vy;
            if (tmp < 0.0) tmp = 0.0;
            psi_s[o] = a * pow(tmp + eps, a - 1.0);
        }
}

static inline void relax_pixel(int j, int i, int m, int n, int K, const double *J11,
                               const double *J22, const double *J12, const double *J13,
                               const double *J23, const double *wgt, const double *psi,
                               const double *psi_s, const double *u, const double *v,
                               double *du, double *dv, double ax, double ay, int smooth_nl,
                               double omega)
{
    (void)m;
    size_t c = (size_t)j * n + i;
    size_t L = c - 1, R = c + 1, D = c + n, U = c - n;
    double den_u = 0, den_v = 0, num_u = 0, num_v = 0, t;
    if (smooth_nl) {
        t = 0.5 * (psi_s[c] + psi_s[L]) * ax;
        num_u += t * (u[L] + du[L] - u[c]); num_v += t * (v[L] + dv[L] - v[c]); den_u += t; den_v += t;
        t = 0.5 * (psi_s[c] + psi_s[R]) * ax;
        num_u += t * (u[R] + du[R] - u[c]); num_v += t * (v[R] + dv[R] - v[c]); den_u += t; den_v += t;
        t = 0.5 * (psi_s[c] + psi_s[D]) * ay;
        num_u += t * (u[D] + du[D] - u[c]); num_v += t * (v[D] + dv[D] - v[c]); den_u += t; den_v += t;
        t = 0.5 * (psi_s[c] + psi_s[U]) * ay;
        num_u += t * (u[U] + du[U] - u[c]); num_v += t * (v[U] + dv[U] - v[c]); den_u += t; den_v += t;
    } else {
        t = ax;
        num_u += t * (u[L] + du[L] - u[c]); num_v += t * (v[L] + dv[L] - v[c]); den_u += t; den_v += t;
        num_u += t * (u[R] + du[R] - u[c]); num_v += t * (v[R] + dv[R] - v[c]); den_u += t; den_v += t;
        t = ay;
        num_u += t * (u[D] + du[D] - u[c]); num_v += t * (v[D] + dv[D] - v[c]); den_u += t; den_v += t;
        num_u += t * (u[U] + du[U] - u[c]); num_v += t * (v[U] + dv[U] - v[c]); den_u += t; den_v += t;
    }
    for (int k = 0; k < K; ++k) {
        size_t ck = c * K + k;
        double wp = wgt[ck] * psi[ck];
        num_u -= wp * (J13[ck] + J12[ck] * dv[c]);
        den_u += wp * J11[ck];
        den_v += wp * J22[ck];
    }
    double du_kp1 = den_u != 0.0 ? num_u / den_u : 0.0;
    du[c] = (1.0 - omega) * du[c] + omega * du_kp1;
    double num_v2 = num_v;
    for (int k = 0; k < K; ++k) {
        size_t ck = c * K + k;
        num_v2 -= wgt[ck] * psi[ck] * (J23[ck] + J12[ck] * du[c]);
    }
    double dv_kp1 = den_v != 0.0 ? num_v2 / den_v : 0.0;
    dv[c] = (1.0 - omega) * dv[c] + omega * dv_kp1;
}

/* gnc_beta < 0: compute_flow (core/level_solver.py:158-369); gnc_beta in [0, 1]:
 * compute_flow_gnc (core/level_solver.py:372-555), which mixes psi and psi_s with the
 * quadratic penalty, (1 - beta) + beta * robust, where the exponent lies in (0, 1). */
int orc_compute_flow(const double *J11, const double *J22, const double *J33, const double *J12,
                     const double *J13, const double *J23, const double *wgt, const double *u,
                     const double *v, int m, int n, int K, double alpha_x, double alpha_y,
                     int iterations, int update_lag, const double *a_data, double a_smooth,
                     double hx, double hy, int order, double omega, double gnc_beta, double *du, double *dv)
{
    const int gnc = gnc_beta >= 0.0;
    const double mix_quadratic = 1.0 - gnc_beta;
    size_t N = (size_t)m * n;
    double *psi = malloc(N * K * sizeof(double));
    double *psi_s = malloc(N * sizeof(double));
    double *scratch = malloc(2 * N * sizeof(double));
    if (!psi || !psi_s || !scratch) { free(psi); free(psi_s); free(scratch); return ORC_ENOMEM; }
    for (size_t i = 0; i < N * K; ++i) psi[i] = 1.0;
    for (size_t i = 0; i < N; ++i) { psi_s[i] = 1.0; du[i] = 0.0; dv[i] = 0.0; }
    const int smooth_nl = a_smooth != 1.0;
    const double ax = alpha_x / (hx * hx), ay = alpha_y / (hy * hy);

    for (int it = 0; it < iterations; ++it) {
        if ((it + 1) % update_lag == 0) {
            /* core/level_solver.py:230-246 (J23*dv appears twice, as in the reference) */
            for (int k = 0; k < K; ++k)
                for (size_t c = 0; c < N; ++c) {
                    size_t ck = c * K + k;
                    double a = du[c], b = dv[c];
                    double val = J11[ck] * a * a + J22[ck] * b * b + J23[ck] * b
                               + 2.0 * J12[ck] * a * b + 2.0 * J13[ck] * a + J23[ck] * b + J33[ck];
                    if (val < 0.0) val = 0.0;
                    const double robust = a_data[k] * pow(val + 0.00001, a_data[k] - 1.0);
                    const int mix = gnc && 0.0 < a_data[k] && a_data[k] < 1.0 && gnc_beta < 1.0;
                    psi[ck] = mix ? mix_quadratic + gnc_beta * robust : robust;
                }
            if (smooth_nl) {
                nonlinearity_smoothness_2d(psi_s, u, du, v, dv, m, n, a_smooth, hx, hy, scratch);
                if (gnc && 0.0 < a_smooth && a_smooth < 1.0 && gnc_beta < 1.0)
                    for (size_t c = 0; c < N; ++c) psi_s[c] = mix_quadratic + gnc_beta * psi_s[c];
            } else
                for (size_t c = 0; c < N; ++c) psi_s[c] = 1.0;
        }
        set_boundary_2d(du, m, n);
        set_boundary_2d(dv, m, n);
        if (order == 0) {
            for (int i = 1; i < n - 1; ++i)
                for (int j = 1; j < m - 1; ++j)
                    relax_pixel(j, i, m, n, K, J11, J22, J12, J13, J23, wgt, psi, psi_s, u, v,
                                du, dv, ax, ay, smooth_nl, omega);
        } else {
            for (int colour = 0; colour < 2; ++colour)
                for (int i = 1; i < n - 1; ++i)
                    for (int j = 1; j < m - 1; ++j)
                        if (((i + j) & 1) == colour)
                            relax_pixel(j, i, m, n, K, J11, J22, J12, J13, J23, wgt, psi, psi_s,
                                        u, v, du, dv, ax, ay, smooth_nl, omega);
        }
    }
    free(psi); free(psi_s); free(scratch);
    return ORC_OK;
}

/* compute_flow (core/level_solver.py:158-369) for a_smooth = 1 in lexicographic
 * order, with every solver value held and every operation rounded in float32
 * (numpy float32 semantics: no fused multiply-add, powf, IEEE division): the
 * reference algorithm in single precision.  Its distance from the float64
 * solver is the rounding envelope of a float32 implementation.  Inputs and the
 * returned du, dv are float64 arrays; the values are rounded to float32 on
 * entry. */
int orc_compute_flow_f32(const double *J11d, const double *J22d, const double *J33d, const double *J12d,
                         const double *J13d, const double *J23d, const double *wgtd, const double *ud,
                         const double *vd, int m, int n, int K, double alpha_x, double alpha_y,
                         int iterations, int update_lag, const double *a_data, double hx, double hy,
                         double omega_d, double *du_out, double *dv_out)
{
    size_t N = (size_t)m * n, NK = N * K;
    float *buf = malloc((7 * NK + 4 * N) * sizeof(float));
    if (!buf) return ORC_ENOMEM;
    float *J11 = buf, *J22 = J11 + NK, *J33 = J22 + NK, *J12 = J33 + NK, *J13 = J12 + NK, *J23 = J13 + NK;
    float *wgt = J23 + NK, *u = wgt + NK, *v = u + N, *du = v + N, *dv = du + N;
    float *psi = malloc(NK * sizeof(float));
    if (!psi) { free(buf); return ORC_ENOMEM; }
    for (size_t i = 0; i < NK; ++i) {
        J11[i] = (float)J11d[i]; J22[i] = (float)J22d[i]; J33[i] = (float)J33d[i];
        J12[i] = (float)J12d[i]; J13[i] = (float)J13d[i]; J23[i] = (float)J23d[i];
        wgt[i] = (float)wgtd[i]; psi[i] = 1.0f;
    }
    for (size_t i = 0; i < N; ++i) { u[i] = (float)ud[i]; v[i] = (float)vd[i]; du[i] = 0.0f; dv[i] = 0.0f; }
    const float ax = (float)(alpha_x / (hx * hx)), ay = (float)(alpha_y / (hy * hy));
    const float omega = (float)omega_d;
    for (int it = 0; it < iterations; ++it) {
        if ((it + 1) % update_lag == 0) {
            for (int k = 0; k < K; ++k) {
                const float ak = (float)a_data[k];
                for (size_t c = 0; c < N; ++c) {
                    size_t ck = c * K + k;
                    float a = du[c], b = dv[c];
                    float val = J11[ck] * a * a + J22[ck] * b * b + J23[ck] * b
                              + 2.0f * J12[ck] * a * b + 2.0f * J13[ck] * a + J23[ck] * b + J33[ck];
                    if (val < 0.0f) val = 0.0f;
                    psi[ck] = ak * powf(val + 0.00001f, ak - 1.0f);
                }
            }
        }
        for (int i = 0; i < n; ++i) {
            du[i] = du[n + i]; du[(size_t)(m - 1) * n + i] = du[(size_t)(m - 2) * n + i];
            dv[i] = dv[n + i]; dv[(size_t)(m - 1) * n + i] = dv[(size_t)(m - 2) * n + i];
        }
        for (int j = 0; j < m; ++j) {
            du[(size_t)j * n] = du[(size_t)j * n + 1]; du[(size_t)j * n + n - 1] = du[(size_t)j * n + n - 2];
            dv[(size_t)j * n] = dv[(size_t)j * n + 1]; dv[(size_t)j * n + n - 1] = dv[(size_t)j * n + n - 2];
        }
        for (int i = 1; i < n - 1; ++i)
            for (int j = 1; j < m - 1; ++j) {
                size_t c = (size_t)j * n + i;
                size_t L = c - 1, R = c + 1, D = c + n, U = c - n;
                float den_u = 0, den_v = 0, num_u = 0, num_v = 0;
                num_u += ax * (u[L] + du[L] - u[c]); num_v += ax * (v[L] + dv[L] - v[c]); den_u += ax; den_v += ax;
                num_u += ax * (u[R] + du[R] - u[c]); num_v += ax * (v[R] + dv[R] - v[c]); den_u += ax; den_v += ax;
                num_u += ay * (u[D] + du[D] - u[c]); num_v += ay * (v[D] + dv[D] - v[c]); den_u += ay; den_v += ay;
                num_u += ay * (u[U] + du[U] - u[c]); num_v += ay * (v[U] + dv[U] - v[c]); den_u += ay; den_v += ay;
                for (int k = 0; k < K; ++k) {
                    size_t ck = c * K + k;
                    float wp = wgt[ck] * psi[ck];
                    num_u -= wp * (J13[ck] + J12[ck] * dv[c]);
                    den_u += wp * J11[ck];
                    den_v += wp * J22[ck];
                }
                float du_kp1 = den_u != 0.0f ? num_u / den_u : 0.0f;
                du[c] = (1.0f - omega) * du[c] + omega * du_kp1;
                float num_v2 = num_v;
                for (int k = 0; k < K; ++k) {
                    size_t ck = c * K + k;
                    num_v2 -= wgt[ck] * psi[ck] * (J23[ck] + J12[ck] * du[c]);
                }
                float dv_kp1 = den_v != 0.0f ? num_v2 / den_v : 0.0f;
                dv[c] = (1.0f - omega) * dv[c] + omega * dv_kp1;
            }
    }
    for (size_t i = 0; i < N; ++i) { du_out[i] = du[i]; dv_out[i] = dv[i]; }
    free(psi); free(buf);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* 5x5 median, scipy.ndimage "mirror" boundary: core/optical_flow.py:607-609 */
/* ------------------------------------------------------------------------ */
static inline int mirror_idx(int i, int n)
{
    if (n == 1) return 0;
    while (i < 0 || i >= n) {
        if (i < 0) i = -i;
        if (i >= n) i = 2 * (n - 1) - i;
    }
    return i;
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

void orc_median5_plane(const double *src, int h, int w, double *dst)
{
    double win[25];
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int q = 0;
            for (int dy = -2; dy <= 2; ++dy) {
                int yy = mirror_idx(y + dy, h);
                for (int dx = -2; dx <= 2; ++dx) win[q++] = src[(size_t)yy * w + mirror_idx(x + dx, w)];
            }
            qsort(win, 25, sizeof(double), cmp_double);
            dst[(size_t)y * w + x] = win[12];
        }
}

/* ------------------------------------------------------------------------ */
/* Full single-stage pyramid: core/optical_flow.py:476-617, 773-929.         */
/* ------------------------------------------------------------------------ */
typedef struct {
    int h, w;                    /* level size (rows, cols) */
    int p_img;                   /* taps of the full-res -> level resize */
    const int32_t *ix_img, *iy_img;
    const float *wx_img, *wy_img;
    int fh, fw;                  /* flow source size (previous level, or full res at the top) */
    int p_flow;
    const int32_t *ix_flow, *iy_flow;
    const float *wx_flow, *wy_flow;
    double alpha_x, alpha_y;     /* alpha with the level scaling applied */
    int top;                     /* 1 for the coarsest level (no warp) */
} orc_level;

typedef struct {
    int iterations, update_lag;
    double a_smooth;
    int gray;                    /* 0: gradient constancy, 1: gray-value constancy, 2: census */
    int order;                   /* 0 lexicographic (numba), 1 red-black */
    double omega;
    int acc_f32;                 /* resize accumulator: 0 float64 (numba), 1 float32 (plain Python) */
    double gnc_beta;             /* < 0: plain stage; else one GNC stage with this beta */
    int warping_steps;           /* warp / relinearise steps per level of a GNC stage */
    int solver_f32;              /* 1: the level solver in float32 (orc_compute_flow_f32; a_smooth = 1,
                                    lexicographic order) */
} orc_params;

/* resize an (H, W, K) double array, channel by channel, to (h, w, K) */
static int resize_hwk(const double *src, int H, int W, int K, double *dst, int h, int w,
                      const int32_t *ix, const float *wx, const int32_t *iy, const float *wy, int P,
                      int acc_f32)
{
    float *plane = malloc((size_t)H * W * sizeof(float));
    float *tmp = malloc((size_t)H * w * sizeof(float));
    float *out = malloc((size_t)h * w * sizeof(float));
    if (!plane || !tmp || !out) { free(plane); free(tmp); free(out); return ORC_ENOMEM; }
    for (int k = 0; k < K; ++k) {
        for (size_t i = 0; i < (size_t)H * W; ++i) plane[i] = (float)src[i * K + k];
        orc_resize_plane(plane, H, W, out, h, w, ix, wx, P, iy, wy, P, tmp, acc_f32);
        for (size_t i = 0; i < (size_t)h * w; ++i) dst[i * K + k] = (double)out[i];
    }
    free(plane); free(tmp); free(out);
    return ORC_OK;
}

static void add_boundary(const double *f, int h, int w, double *p)
{
    pad1_d(f, h, w, p);
}

int orc_displacement(int H, int W, int K, const double *fixed, const double *moving,
                     const double *weight, const double *uv, int n_levels,
                     const orc_level *levels, const double *a_data, const orc_params *prm,
                     double *w_out /* h_last * w_last * 2 */)
{
    int rc = ORC_OK;
    double *u = NULL, *v = NULL; /* padded current flow */
    int ph = 0, pw = 0;          /* interior size of u, v */
    size_t full = (size_t)H * W;
    double *u_init = malloc(full * sizeof(double)), *v_init = malloc(full * sizeof(double));
    if (!u_init || !v_init) { free(u_init); free(v_init); return ORC_ENOMEM; }
    for (size_t i = 0; i < full; ++i) {
        u_init[i] = uv ? uv[i * 2 + 0] : 0.0;
        v_init[i] = uv ? uv[i * 2 + 1] : 0.0;
    }
    for (int li = 0; li < n_levels && rc == ORC_OK; ++li) {
        const orc_level *L = &levels[li];
        int h = L->h, w = L->w, m = h + 2, n = w + 2;
        size_t hw = (size_t)h * w, mn = (size_t)m * n;
        double *f1 = malloc(hw * K * sizeof(double)), *f2 = malloc(hw * K * sizeof(double));
        double *wl = malloc(hw * K * sizeof(double));
        double *ur = malloc(hw * sizeof(double)), *vr = malloc(hw * sizeof(double));
        double *un = malloc(mn * sizeof(double)), *vn = malloc(mn * sizeof(double));
        double *tmp = malloc(hw * K * sizeof(double));
        double *J = malloc(6 * mn * K * sizeof(double));
        double *Jc = malloc(6 * mn * sizeof(double));
        double *wpad = malloc(mn * K * sizeof(double));
        double *du = malloc(mn * sizeof(double)), *dv = malloc(mn * sizeof(double));
        double *plane1 = malloc(hw * sizeof(double)), *plane2 = malloc(hw * sizeof(double));
        double *uw = malloc(hw * sizeof(double)), *vw = malloc(hw * sizeof(double));
        float *wf = malloc(hw * sizeof(float));
        double *med = malloc(hw * sizeof(double)), *medo = malloc(hw * sizeof(double));
        if (!f1 || !f2 || !wl || !ur || !vr || !un || !vn || !tmp || !J || !Jc || !wpad || !du ||
            !dv || !plane1 || !plane2 || !uw || !vw || !wf || !med || !medo) {
            rc = ORC_ENOMEM;
        }
        if (rc == ORC_OK) {
            /* pyramid images from full resolution (lines 519-520) */
            rc = resize_hwk(fixed, H, W, K, f1, h, w, L->ix_img, L->wx_img, L->iy_img, L->wy_img, L->p_img, prm->acc_f32);
            if (rc == ORC_OK)
                rc = resize_hwk(moving, H, W, K, f2, h, w, L->ix_img, L->wx_img, L->iy_img, L->wy_img, L->p_img, prm->acc_f32);
        }
        double h_row = (double)H / h, h_col = (double)W / w;
        if (rc == ORC_OK) {
            /* flow to this level (lines 530-536) */
            const double *su = L->top ? u_init : NULL, *sv = L->top ? v_init : NULL;
            double *iu = NULL, *iv = NULL;
            if (!L->top) {
                iu = malloc((size_t)ph * pw * sizeof(double));
                iv = malloc((size_t)ph * pw * sizeof(double));
                if (!iu || !iv) rc = ORC_ENOMEM;
                else {
                    for (int y = 0; y < ph; ++y)
                        for (int x = 0; x < pw; ++x) {
                            iu[(size_t)y * pw + x] = u[(size_t)(y + 1) * (pw + 2) + x + 1];
                            iv[(size_t)y * pw + x] = v[(size_t)(y + 1) * (pw + 2) + x + 1];
                        }
                    su = iu; sv = iv;
                }
            }
            if (rc == ORC_OK) rc = resize_hwk(su, L->fh, L->fw, 1, ur, h, w, L->ix_flow, L->wx_flow, L->iy_flow, L->wy_flow, L->p_flow, prm->acc_f32);
            if (rc == ORC_OK) rc = resize_hwk(sv, L->fh, L->fw, 1, vr, h, w, L->ix_flow, L->wx_flow, L->iy_flow, L->wy_flow, L->p_flow, prm->acc_f32);
            free(iu); free(iv);
        }
        if (rc == ORC_OK) {
            add_boundary(ur, h, w, un);
            add_boundary(vr, h, w, vn);
            /* warp (lines 533-544) */
            if (L->top) {
                memcpy(tmp, f2, hw * K * sizeof(double));
            } else {
                for (size_t i = 0; i < hw; ++i) {
                    int y = (int)(i / w), x = (int)(i % w);
                    uw[i] = un[(size_t)(y + 1) * n + x + 1] / h_col;
                    vw[i] = vn[(size_t)(y + 1) * n + x + 1] / h_row;
                }
                for (int k = 0; k < K; ++k) {
                    for (size_t i = 0; i < hw; ++i) { plane1[i] = f1[i * K + k]; plane2[i] = f2[i * K + k]; }
                    orc_warp_plane(plane2, plane1, uw, vw, h, w, 1, wf);
                    for (size_t i = 0; i < hw; ++i) tmp[i * K + k] = (double)wf[i];
                }
            }
            /* motion tensor per channel (lines 547-563) */
            for (int k = 0; k < K && rc == ORC_OK; ++k) {
                for (size_t i = 0; i < hw; ++i) { plane1[i] = f1[i * K + k]; plane2[i] = tmp[i * K + k]; }
                rc = orc_motion_tensor(plane1, plane2, h, w, h_row, h_col, !L->top, prm->gray,
                                       Jc, Jc + mn, Jc + 2 * mn, Jc + 3 * mn, Jc + 4 * mn, Jc + 5 * mn);
                for (int q = 0; q < 6; ++q)
                    for (size_t i = 0; i < mn; ++i) J[(size_t)q * mn * K + i * K + k] = Jc[(size_t)q * mn + i];
            }
        }
        if (rc == ORC_OK) {
            /* weight level with a zero ring (lines 565-570) */
            rc = resize_hwk(weight, H, W, K, wl, h, w, L->ix_img, L->wx_img, L->iy_img, L->wy_img, L->p_img, prm->acc_f32);
            memset(wpad, 0, mn * K * sizeof(double));
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x)
                    for (int k = 0; k < K; ++k)
                        wpad[((size_t)(y + 1) * n + x + 1) * K + k] = wl[((size_t)y * w + x) * K + k];
        }
        if (rc == ORC_OK) {
            /* level solve (lines 584-606): hx = h_col, hy = h_row */
            if (prm->solver_f32)
                rc = (prm->a_smooth != 1.0 || prm->order != 0) ? ORC_EINVAL
                   : orc_compute_flow_f32(J, J + mn * K, J + 2 * mn * K, J + 3 * mn * K, J + 4 * mn * K,
                                          J + 5 * mn * K, wpad, un, vn, m, n, K, L->alpha_x, L->alpha_y,
                                          prm->iterations, prm->update_lag, a_data, h_col, h_row,
                                          prm->omega, du, dv);
            else
                rc = orc_compute_flow(J, J + mn * K, J + 2 * mn * K, J + 3 * mn * K, J + 4 * mn * K,
                                      J + 5 * mn * K, wpad, un, vn, m, n, K, L->alpha_x, L->alpha_y,
                                      prm->iterations, prm->update_lag, a_data, prm->a_smooth,
                                      h_col, h_row, prm->order, prm->omega, -1.0, du, dv);
        }
        if (rc == ORC_OK) {
            /* median on the interiors (lines 607-609), then accumulate (610-611) */
            if ((h < w ? h : w) > 5) {
                for (int pass = 0; pass < 2; ++pass) {
                    double *d = pass == 0 ? du : dv;
                    for (int y = 0; y < h; ++y)
                        for (int x = 0; x < w; ++x) med[(size_t)y * w + x] = d[(size_t)(y + 1) * n + x + 1];
                    orc_median5_plane(med, h, w, medo);
                    for (int y = 0; y < h; ++y)
                        for (int x = 0; x < w; ++x) d[(size_t)(y + 1) * n + x + 1] = medo[(size_t)y * w + x];
                }
            }
            for (size_t i = 0; i < mn; ++i) { un[i] += du[i]; vn[i] += dv[i]; }
            free(u); free(v);
            u = un; v = vn; un = NULL; vn = NULL;
            ph = h; pw = w;
        }
        free(f1); free(f2); free(wl); free(ur); free(vr); free(un); free(vn); free(tmp); free(J);
        free(Jc); free(wpad); free(du); free(dv); free(plane1); free(plane2); free(uw); free(vw);
        free(wf); free(med); free(medo);
    }
    if (rc == ORC_OK) {
        for (int y = 0; y < ph; ++y)
            for (int x = 0; x < pw; ++x) {
                w_out[((size_t)y * pw + x) * 2 + 0] = u[(size_t)(y + 1) * (pw + 2) + x + 1];
                w_out[((size_t)y * pw + x) * 2 + 1] = v[(size_t)(y + 1) * (pw + 2) + x + 1];
            }
    }
    free(u); free(v); free(u_init); free(v_init);
    return rc;
}

/* One GNC stage (core/optical_flow.py:620-770): per level, warping_steps rounds of
 * warp (every level, the top one included, so the warped frame is always float32),
 * tensor, compute_flow_gnc from du = dv = 0, u += du, and a 5x5 median of u itself. */
int orc_displacement_gnc(int H, int W, int K, const double *fixed, const double *moving,
                         const double *weight, const double *uv, int n_levels,
                         const orc_level *levels, const double *a_data, const orc_params *prm,
                         double *w_out)
{
    int rc = ORC_OK;
    double *u = NULL, *v = NULL;
    int ph = 0, pw = 0;
    size_t full = (size_t)H * W;
    double *u_init = malloc(full * sizeof(double)), *v_init = malloc(full * sizeof(double));
    if (!u_init || !v_init) { free(u_init); free(v_init); return ORC_ENOMEM; }
    for (size_t i = 0; i < full; ++i) {
        u_init[i] = uv ? uv[i * 2 + 0] : 0.0;
        v_init[i] = uv ? uv[i * 2 + 1] : 0.0;
    }
    for (int li = 0; li < n_levels && rc == ORC_OK; ++li) {
        const orc_level *L = &levels[li];
        int h = L->h, w = L->w, m = h + 2, n = w + 2;
        size_t hw = (size_t)h * w, mn = (size_t)m * n;
        double *f1 = malloc(hw * K * sizeof(double)), *f2 = malloc(hw * K * sizeof(double));
        double *wl = malloc(hw * K * sizeof(double));
        double *ur = malloc(hw * sizeof(double)), *vr = malloc(hw * sizeof(double));
        double *un = malloc(mn * sizeof(double)), *vn = malloc(mn * sizeof(double));
        double *tmp = malloc(hw * K * sizeof(double));
        double *J = malloc(6 * mn * K * sizeof(double));
        double *Jc = malloc(6 * mn * sizeof(double));
        double *wpad = malloc(mn * K * sizeof(double));
        double *du = malloc(mn * sizeof(double)), *dv = malloc(mn * sizeof(double));
        double *plane1 = malloc(hw * sizeof(double)), *plane2 = malloc(hw * sizeof(double));
        double *uw = malloc(hw * sizeof(double)), *vw = malloc(hw * sizeof(double));
        float *wf = malloc(hw * sizeof(float));
        double *med = malloc(hw * sizeof(double)), *medo = malloc(hw * sizeof(double));
        if (!f1 || !f2 || !wl || !ur || !vr || !un || !vn || !tmp || !J || !Jc || !wpad || !du ||
            !dv || !plane1 || !plane2 || !uw || !vw || !wf || !med || !medo)
            rc = ORC_ENOMEM;
        if (rc == ORC_OK)
            rc = resize_hwk(fixed, H, W, K, f1, h, w, L->ix_img, L->wx_img, L->iy_img, L->wy_img, L->p_img, prm->acc_f32);
        if (rc == ORC_OK)
            rc = resize_hwk(moving, H, W, K, f2, h, w, L->ix_img, L->wx_img, L->iy_img, L->wy_img, L->p_img, prm->acc_f32);
        double h_row = (double)H / h, h_col = (double)W / w;
        if (rc == ORC_OK) {
            const double *su = L->top ? u_init : NULL, *sv = L->top ? v_init : NULL;
            double *iu = NULL, *iv = NULL;
            if (!L->top) {
                iu = malloc((size_t)ph * pw * sizeof(double));
                iv = malloc((size_t)ph * pw * sizeof(double));
                if (!iu || !iv) rc = ORC_ENOMEM;
                else {
                    for (int y = 0; y < ph; ++y)
                        for (int x = 0; x < pw; ++x) {
                            iu[(size_t)y * pw + x] = u[(size_t)(y + 1) * (pw + 2) + x + 1];
                            iv[(size_t)y * pw + x] = v[(size_t)(y + 1) * (pw + 2) + x + 1];
                        }
                    su = iu; sv = iv;
                }
            }
            if (rc == ORC_OK) rc = resize_hwk(su, L->fh, L->fw, 1, ur, h, w, L->ix_flow, L->wx_flow, L->iy_flow, L->wy_flow, L->p_flow, prm->acc_f32);
            if (rc == ORC_OK) rc = resize_hwk(sv, L->fh, L->fw, 1, vr, h, w, L->ix_flow, L->wx_flow, L->iy_flow, L->wy_flow, L->p_flow, prm->acc_f32);
            free(iu); free(iv);
        }
        if (rc == ORC_OK) {
            add_boundary(ur, h, w, un);
            add_boundary(vr, h, w, vn);
            rc = resize_hwk(weight, H, W, K, wl, h, w, L->ix_img, L->wx_img, L->iy_img, L->wy_img, L->p_img, prm->acc_f32);
            memset(wpad, 0, mn * K * sizeof(double));
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x)
                    for (int k = 0; k < K; ++k)
                        wpad[((size_t)(y + 1) * n + x + 1) * K + k] = wl[((size_t)y * w + x) * K + k];
        }
        for (int ws = 0; ws < prm->warping_steps && rc == ORC_OK; ++ws) {
            for (size_t i = 0; i < hw; ++i) {
                int y = (int)(i / w), x = (int)(i % w);
                uw[i] = un[(size_t)(y + 1) * n + x + 1] / h_col;
                vw[i] = vn[(size_t)(y + 1) * n + x + 1] / h_row;
            }
            for (int k = 0; k < K; ++k) {
                for (size_t i = 0; i < hw; ++i) { plane1[i] = f1[i * K + k]; plane2[i] = f2[i * K + k]; }
                orc_warp_plane(plane2, plane1, uw, vw, h, w, 1, wf);
                for (size_t i = 0; i < hw; ++i) tmp[i * K + k] = (double)wf[i];
            }
            for (int k = 0; k < K && rc == ORC_OK; ++k) {
                for (size_t i = 0; i < hw; ++i) { plane1[i] = f1[i * K + k]; plane2[i] = tmp[i * K + k]; }
                rc = orc_motion_tensor(plane1, plane2, h, w, h_row, h_col, 1, prm->gray,
                                       Jc, Jc + mn, Jc + 2 * mn, Jc + 3 * mn, Jc + 4 * mn, Jc + 5 * mn);
                for (int q = 0; q < 6; ++q)
                    for (size_t i = 0; i < mn; ++i) J[(size_t)q * mn * K + i * K + k] = Jc[(size_t)q * mn + i];
            }
            if (rc == ORC_OK)
                rc = orc_compute_flow(J, J + mn * K, J + 2 * mn * K, J + 3 * mn * K, J + 4 * mn * K,
                                      J + 5 * mn * K, wpad, un, vn, m, n, K, L->alpha_x, L->alpha_y,
                                      prm->iterations, prm->update_lag, a_data, prm->a_smooth,
                                      h_col, h_row, prm->order, prm->omega, prm->gnc_beta, du, dv);
            if (rc == ORC_OK) {
                for (size_t i = 0; i < mn; ++i) { un[i] += du[i]; vn[i] += dv[i]; }
                if ((h < w ? h : w) > 5) {
                    for (int pass = 0; pass < 2; ++pass) {
                        double *d = pass == 0 ? un : vn;
                        for (int y = 0; y < h; ++y)
                            for (int x = 0; x < w; ++x) med[(size_t)y * w + x] = d[(size_t)(y + 1) * n + x + 1];
                        orc_median5_plane(med, h, w, medo);
                        add_boundary(medo, h, w, d);
                    }
                }
            }
        }
        if (rc == ORC_OK) {
            free(u); free(v);
            u = un; v = vn; un = NULL; vn = NULL;
            ph = h; pw = w;
        }
        free(f1); free(f2); free(wl); free(ur); free(vr); free(un); free(vn); free(tmp); free(J);
        free(Jc); free(wpad); free(du); free(dv); free(plane1); free(plane2); free(uw); free(vw);
        free(wf); free(med); free(medo);
    }
    if (rc == ORC_OK) {
        for (int y = 0; y < ph; ++y)
            for (int x = 0; x < pw; ++x) {
                w_out[((size_t)y * pw + x) * 2 + 0] = u[(size_t)(y + 1) * (pw + 2) + x + 1];
                w_out[((size_t)y * pw + x) * 2 + 1] = v[(size_t)(y + 1) * (pw + 2) + x + 1];
            }
    }
    free(u); free(v); free(u_init); free(v_init);
    return rc;
}

/* Many frames against one reference, parallel over frames with OpenMP.
 * fixed: (H, W, K); moving: (T, H, W, K); out: (T, h_last, w_last, 2). */
int orc_displacement_batch(int T, int H, int W, int K, const double *fixed, const double *moving,
                           const double *weight, const double *uv, int n_levels,
                           const orc_level *levels, const double *a_data, const orc_params *prm,
                           int out_h, int out_w, double *w_out, int n_threads)
{
    int rc_all = ORC_OK;
    size_t fsz = (size_t)H * W * K, osz = (size_t)out_h * out_w * 2;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
#endif
    for (int t = 0; t < T; ++t) {
        int rc = orc_displacement(H, W, K, fixed, moving + (size_t)t * fsz, weight, uv, n_levels,
                                  levels, a_data, prm, w_out + (size_t)t * osz);
        if (rc != ORC_OK) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
            rc_all = rc;
        }
    }
    (void)n_threads;
    return rc_all;
}
