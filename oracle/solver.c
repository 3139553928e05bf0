/*
 * CPU oracle for the evaluation path: the reference solver and the scoring
 * metrics. TEST INFRASTRUCTURE ONLY (see oracle.h): the checker that the
 * library's CUDA solver and metrics are compared against, and the timed CPU
 * baseline of the evaluation. Never linked into the product.
 *
 * Restates, in f32 with the reference's operation order and no fused
 * multiply-add (built with -ffp-contract=off):
 *   crates/solvers/src/shallow_water.rs:102-111   State::add_drop
 *   crates/solvers/src/shallow_water.rs:114-124   mirror (ghost cells)
 *   crates/solvers/src/shallow_water.rs:149-238   ShallowWater::step
 *   crates/engine/src/norm.rs:27-34               Normalizer::encode
 *   crates/engine/src/metrics.rs:9-112            correlation, peak, mean,
 *                                                 std_dev, bias,
 *                                                 radial_profile, xcorr_lag,
 *                                                 decode_h, rmse
 *   crates/engine-cli/src/eval.rs:158-171         one scored row
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* shallow_water.rs:116-124 */
static int mirror(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

void orc_sw_add_drop(const orc_sw_params* p, float* h, float cx, float cy, float amp, float sigma) {
    const float inv = 1.0f / (2.0f * sigma * sigma);
    for (int y = 0; y < p->ny; y++)
        for (int x = 0; x < p->nx; x++) {
            const float dx = (float)x - cx, dy = (float)y - cy;
            h[y * p->nx + x] += amp * expf(-(dx * dx + dy * dy) * inv);
        }
}

double orc_sw_mass(const float* h, int n) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += (double)h[i];
    return s;
}

/* shallow_water.rs:149-238. `work` holds (nx+1)*ny + nx*(ny+1) + 3*nx*ny
 * floats, or is NULL (allocated here). */
static void sw_step(const orc_sw_params* p, float* h, float* u, float* v, float* work) {
    const int nx = p->nx, ny = p->ny, n = nx * ny;
    float* fx = work;
    float* fy = fx + (size_t)(nx + 1) * ny;
    float* hn = fy + (size_t)nx * (ny + 1);
    float* un = hn + n;
    float* vn = un + n;
    for (int y = 0; y < ny; y++) {
        for (int x = 1; x < nx; x++) {
            const int a = y * nx + x - 1, b = y * nx + x;
            fx[y * (nx + 1) + x] = 0.5f * (h[a] + h[b]) * 0.5f * (u[a] + u[b]);
        }
        fx[y * (nx + 1)] = 0.0f;
        fx[y * (nx + 1) + nx] = 0.0f;
    }
    for (int x = 0; x < nx; x++) {
        for (int y = 1; y < ny; y++) {
            const int a = (y - 1) * nx + x, b = y * nx + x;
            fy[y * nx + x] = 0.5f * (h[a] + h[b]) * 0.5f * (v[a] + v[b]);
        }
        fy[x] = 0.0f;
        fy[ny * nx + x] = 0.0f;
    }
    const float r = p->dt / p->dx;
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const float dfx = fx[y * (nx + 1) + x + 1] - fx[y * (nx + 1) + x];
            const float dfy = fy[(y + 1) * nx + x] - fy[y * nx + x];
            hn[y * nx + x] = h[y * nx + x] - r * (dfx + dfy);
        }
    const float inv2dx = 1.0f / (2.0f * p->dx);
    const float invdx2 = 1.0f / (p->dx * p->dx);
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const int i = y * nx + x;
            const int xm = mirror(x - 1, nx), xp = mirror(x + 1, nx);
            const int ym = mirror(y - 1, ny), yp = mirror(y + 1, ny);
            const float sxm = x == 0 ? -1.0f : 1.0f, sxp = x + 1 == nx ? -1.0f : 1.0f;
            const float sym = y == 0 ? -1.0f : 1.0f, syp = y + 1 == ny ? -1.0f : 1.0f;
            const float hl = hn[y * nx + xm], hr = hn[y * nx + xp];
            const float hd = hn[ym * nx + x], hu = hn[yp * nx + x];
            const float ul = sxm * u[y * nx + xm], ur = sxp * u[y * nx + xp];
            const float ud = u[ym * nx + x], uu = u[yp * nx + x];
            const float vl = v[y * nx + xm], vr = v[y * nx + xp];
            const float vd = sym * v[ym * nx + x], vu = syp * v[yp * nx + x];
            const float u0 = u[i], v0 = v[i];
            const float dudx = (ur - ul) * inv2dx, dudy = (uu - ud) * inv2dx;
            const float dvdx = (vr - vl) * inv2dx, dvdy = (vu - vd) * inv2dx;
            const float dhdx = (hr - hl) * inv2dx, dhdy = (hu - hd) * inv2dx;
            const float lap_u = (ul + ur + ud + uu - 4.0f * u0) * invdx2;
            const float lap_v = (vl + vr + vd + vu - 4.0f * v0) * invdx2;
            un[i] = u0 + p->dt * (-u0 * dudx - v0 * dudy - p->g * dhdx + p->nu * lap_u);
            vn[i] = v0 + p->dt * (-u0 * dvdx - v0 * dvdy - p->g * dhdy + p->nu * lap_v);
        }
    memcpy(h, hn, (size_t)n * 4);
    memcpy(u, un, (size_t)n * 4);
    memcpy(v, vn, (size_t)n * 4);
}

void orc_sw_steps(const orc_sw_params* p, float* h, float* u, float* v, int steps) {
    const size_t nw = (size_t)(p->nx + 1) * p->ny + (size_t)p->nx * (p->ny + 1) + 3 * (size_t)p->nx * p->ny;
    float* work = (float*)malloc(nw * 4);
    if (!work) return;
    for (int t = 0; t < steps; t++) sw_step(p, h, u, v, work);
    free(work);
}

/* metrics.rs:9-23 */
float orc_correlation(const float* a, const float* b, int n) {
    double sa = 0.0, sb = 0.0;
    for (int i = 0; i < n; i++) sa += (double)a[i];
    for (int i = 0; i < n; i++) sb += (double)b[i];
    const double ma = sa / (double)n, mb = sb / (double)n;
    double sab = 0.0, saa = 0.0, sbb = 0.0;
    for (int i = 0; i < n; i++) {
        const double dx = (double)a[i] - ma, dy = (double)b[i] - mb;
        sab += dx * dy;
        saa += dx * dx;
        sbb += dy * dy;
    }
    if (saa <= 0.0 || sbb <= 0.0) return 0.0f;
    return (float)(sab / sqrt(saa * sbb));
}

/* metrics.rs:25-41 */
float orc_peak(const float* f, int n) {
    float m = 0.0f;
    for (int i = 0; i < n; i++) m = fmaxf(m, fabsf(f[i]));
    return m;
}

float orc_mean(const float* f, int n) {
    float s = 0.0f;
    for (int i = 0; i < n; i++) s += f[i];
    return s / (float)n;
}

float orc_std_dev(const float* f, int n) {
    const float m = orc_mean(f, n);
    float s = 0.0f;
    for (int i = 0; i < n; i++) {
        const float d = f[i] - m;
        s += d * d;
    }
    return sqrtf(s / (float)n);
}

float orc_bias(const float* model, const float* solver, int n) {
    return (orc_mean(model, n) - orc_mean(solver, n)) / fmaxf(orc_std_dev(solver, n), 1e-12f);
}

/* metrics.rs:45-61. Returns the profile length rmax + 1 (at most cap). */
int orc_radial_profile(const float* f, int nx, int ny, float cx, float cy, double* out, int cap) {
    float m = fminf(fminf(fminf(cx, cy), (float)nx - cx), (float)ny - cy);
    m = fmaxf(floorf(m), 1.0f);
    const int rmax = (int)m;
    if (rmax + 1 > cap) return -1;
    unsigned* count = (unsigned*)calloc((size_t)rmax + 1, sizeof(unsigned));
    for (int b = 0; b <= rmax; b++) out[b] = 0.0;
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const float dx = (float)x - cx, dy = (float)y - cy;
            const float r = sqrtf(dx * dx + dy * dy);
            const int bin = (int)(r + 0.5f);
            if (bin <= rmax) {
                out[bin] += (double)fabsf(f[y * nx + x]);
                count[bin]++;
            }
        }
    for (int b = 0; b <= rmax; b++) out[b] = count[b] == 0 ? 0.0 : out[b] / (double)count[b];
    free(count);
    return rmax + 1;
}

/* metrics.rs:63-77 */
static float corr_at_lag(const double* model, const double* solver, int n, int lag) {
    float* a = (float*)malloc((size_t)n * 4);
    float* b = (float*)malloc((size_t)n * 4);
    int k = 0;
    for (int i = 0; i < n; i++) {
        const int si = i - lag;
        if (si >= 0 && si < n) {
            a[k] = (float)model[i];
            b[k] = (float)solver[si];
            k++;
        }
    }
    const float c = k < 3 ? -INFINITY : orc_correlation(a, b, k);
    free(a);
    free(b);
    return c;
}

/* metrics.rs:81-101 */
float orc_xcorr_lag(const double* model, const double* solver, int n, int max_lag) {
    int best_lag = 0;
    float best_c = -INFINITY;
    for (int lag = -max_lag; lag <= max_lag; lag++) {
        const float c = corr_at_lag(model, solver, n, lag);
        if (c > best_c) {
            best_c = c;
            best_lag = lag;
        }
    }
    if (best_lag > -max_lag && best_lag < max_lag) {
        const float l = corr_at_lag(model, solver, n, best_lag - 1), c = best_c,
                    r = corr_at_lag(model, solver, n, best_lag + 1);
        if (isfinite(l) && isfinite(r)) {
            const float den = l - 2.0f * c + r;
            if (den < 0.0f) return (float)best_lag + 0.5f * (l - r) / den;
        }
    }
    return (float)best_lag;
}

/* metrics.rs:109-112 */
float orc_rmse(const float* a, const float* b, int n) {
    double s = 0.0;
    for (int i = 0; i < n; i++) {
        const double d = (double)(a[i] - b[i]);
        s += d * d;
    }
    return (float)sqrt(s / (double)n);
}

/* norm.rs:27-34 */
void orc_encode(const float norm_mean[3], const float norm_std[3], float norm_depth, const float* h, const float* u,
                const float* v, int n, float* out) {
    for (int i = 0; i < n; i++) {
        out[i] = (h[i] - norm_depth - norm_mean[0]) / norm_std[0];
        out[n + i] = (u[i] - norm_mean[1]) / norm_std[1];
        out[2 * n + i] = (v[i] - norm_mean[2]) / norm_std[2];
    }
}

/* eval.rs:158-171: one row (corr, corr_h, amplitude ratio, lag, bias) for a
 * normalized model state x [3, ny, nx] against the solver state (h, u, v). */
void orc_eval_score(const float norm_mean[3], const float norm_std[3], float norm_depth, int nx, int ny,
                    const float* x, const float* h, const float* u, const float* v, float cx, float cy,
                    float row[5]) {
    const int n = nx * ny;
    float* target = (float*)malloc((size_t)3 * n * 4);
    float* ph = (float*)malloc((size_t)n * 4);
    float* th = (float*)malloc((size_t)n * 4);
    orc_encode(norm_mean, norm_std, norm_depth, h, u, v, n, target);
    for (int i = 0; i < n; i++) {
        ph[i] = x[i] * norm_std[0] + norm_mean[0];
        th[i] = target[i] * norm_std[0] + norm_mean[0];
    }
    const int cap = nx + ny + 2;
    double* mp = (double*)malloc((size_t)cap * 8);
    double* tp = (double*)malloc((size_t)cap * 8);
    const int len = orc_radial_profile(ph, nx, ny, cx, cy, mp, cap);
    orc_radial_profile(th, nx, ny, cx, cy, tp, cap);
    row[0] = orc_correlation(x, target, 3 * n);
    row[1] = orc_correlation(x, target, n);
    row[2] = orc_peak(ph, n) / orc_peak(th, n);
    row[3] = orc_xcorr_lag(mp, tp, len, 8);
    row[4] = orc_bias(ph, th, n);
    free(target);
    free(ph);
    free(th);
    free(mp);
    free(tp);
}
